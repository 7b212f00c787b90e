// cylqueue.cu — the point-level cylinder fit of a keyframe (cyl_mode 1, and
// the RANSAC fallback pass of cyl_mode 2) as one persistent work-queue
// kernel: inlier counting of the tree's hypotheses, the best hypothesis, and
// the least-squares refinement, over trees of very uneven size.
//
// The reference fits its trees one after the other (sloam.cpp:418-434, one
// Cylinder per landmark).  Here a tree of n points is cut into chunks of
// kC points, and every (phase, tree, chunk) is one work item:
//   phase 0        count the inliers of all K hypotheses on the chunk
//                  (ballot + popcount per 32 points, integer atomics);
//   phase 1..L     one LS iteration: the 20 normal-equation sums of each
//                  256-point slice of the chunk (FP32 per point, warp-shuffle
//                  sums, FP64 across warps).
// Items are numbered phase-major, and within a phase the trees come in
// decreasing size, so that the long chains of the largest trees start first.
// Blocks take items from one atomic counter.  The block that completes the
// last chunk of (tree, phase) finishes the phase for the tree: after phase 0
// the best hypothesis (most inliers, lowest index on ties) and the initial
// model; after an LS phase the slice sums in slice order (FP64, a fixed
// order: the results depend neither on which block ran which chunk nor on
// the chunk size, the hypothesis tile or the block count), the FP64
// 5x5 solve on one warp and the model update; after the last phase the
// cylinder record.  An item of phase p > 0 waits until its tree has
// finished phase p - 1.  Items are claimed in increasing order and a block
// never waits while it holds an unfinished item, so the lowest unfinished
// item always belongs to a running block whose dependencies are done: the
// waits end.  Each wait is still bounded (kQueueWaitPolls); when one runs
// out the kernel sets the counters' error flag and its blocks stop.
#include "cylinder.cuh"
#include "internal.h"
#include "scan_util.cuh"

namespace sg {

namespace {

constexpr int kQThreads = 256;
constexpr int kQWarps = kQThreads / 32;
constexpr int kQSortCap = 4096;           // trees per keyframe the queue orders
constexpr long long kQueueWaitPolls = 1ll << 22;  // x ~100 ns: about 0.4 s

__device__ __forceinline__ bool queue_eligible(const Dev& d, const CylD& c, int l,
                                               const int32_t* only) {
  return c.stage == 1 && c.radius != -1.0 && (!only || only[l]);
}

// One block: the eligible trees with points, ordered by decreasing point
// count (ties by index), their chunk offsets, and the per-tree phase state
// reset.  chunk = points per work item.
__global__ void __launch_bounds__(1024) k_cyl_queue_prep(Dev d, KParams kp,
                                                         const int32_t* __restrict__ only,
                                                         int chunk) {
  __shared__ unsigned long long key[kQSortCap];
  __shared__ int sm[33];
  const int nl = d.cnt->n_lm;
  QueueCtl* q = d.qctl;
  if (nl > kQSortCap) {
    if (threadIdx.x == 0) {
      atomicOr(&d.cnt->overflow, 64);
      q->tc = 0;
      q->nq = 0;
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
  int base = 0, sbase = 0, nq = 0;
  for (int i0 = 0; i0 < n2; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    int nc = 0;
    if (i < n2 && key[i] != ~0ull) {
      const int l = (int)(uint32_t)key[i];
      const int n = (int)(0xFFFFFFFFu - (uint32_t)(key[i] >> 32));
      nc = (n + chunk - 1) / chunk;
      d.q_order[i] = l;
      d.q_ready[l] = 0;
      for (int p = 0; p < P; ++p) d.q_done[(size_t)l * kQueuePhases + p] = 0;
    }
    int total, stotal;
    const int ex = block_excl_scan(nc, sm, &total);
    const int ns = nc ? (int)((0xFFFFFFFFu - (uint32_t)(key[i] >> 32) + 255u) / 256u) : 0;
    const int sex = block_excl_scan(ns, sm, &stotal);
    if (nc) {
      d.q_off[i] = base + ex;
      d.q_soff[i] = sbase + sex;
    }
    base += total;
    sbase += stotal;
    const int cnt = __syncthreads_count(nc > 0);
    nq += cnt;
    // (the last chunk of a tree holds its remainder: points = slices' points)
    if (nc && !only) atomicAdd(&d.cnt->n_fit_pts,
                               (int)(0xFFFFFFFFu - (uint32_t)(key[i] >> 32)));
  }
  if (threadIdx.x == 0) {
    d.q_off[nq] = base;
    d.q_soff[nq] = sbase;
    q->tc = base;
    q->nq = nq;
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

// Dynamic shared memory of the worker: the hypothesis tile, the per-warp
// counts of the tile, then the small state.
template <int kTile>
struct QueueSmem {
  float4 hyp[kTile];
  int cnt[kQWarps][kTile];
};

template <int kPPT, int kTile>
__global__ void __launch_bounds__(kQThreads) k_cyl_queue(Dev d, KParams kp) {
  extern __shared__ __align__(16) unsigned char q_smem[];
  QueueSmem<kTile>& S = *reinterpret_cast<QueueSmem<kTile>*>(q_smem);
  __shared__ float red[20][kQWarps];
  __shared__ double st[16];  // c(3), dir(3), r, ok, b1(3), b2(3), best count, best h
  __shared__ double ssum[20];
  __shared__ double sxls[5];
  __shared__ unsigned long long sk[kQWarps];
  __shared__ int s_idx, s_last, s_stop;
  constexpr int kC = kPPT * kQThreads;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  QueueCtl* q = d.qctl;
  const int TC = q->tc, P = q->phases, nq = q->nq, K = kp.K;
  const long long total = (long long)TC * P;
  for (;;) {
    if (tid == 0) {
      s_idx = atomicAdd(&q->head, 1);
      s_stop = 0;
    }
    __syncthreads();
    const int idx = s_idx;
    if ((long long)idx >= total) break;  // block-uniform
    const int p = idx / TC, r = idx - p * TC;
    int lo = 0, hi = nq - 1;  // the tree whose chunks hold r
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (d.q_off[mid] <= r) lo = mid;
      else hi = mid - 1;
    }
    const int l = d.q_order[lo], c0 = d.q_off[lo], nc = d.q_off[lo + 1] - c0, c = r - c0;
    const int s0 = d.q_soff[lo], ns = d.q_soff[lo + 1] - s0;  // 256-point slices
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
            s_stop = 1;
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
      }
      __syncthreads();
      if (s_stop) break;
    }
    if (p == 0) {
      // ---- inlier counts of the chunk for every hypothesis of the tree
      float2 pu[kPPT];
      bool mine[kPPT];
#pragma unroll
      for (int k = 0; k < kPPT; ++k) {
        const int i = c * kC + k * kQThreads + tid;
        mine[k] = i < n;
        pu[k] = mine[k] ? uvs[i] : make_float2(0.f, 0.f);
      }
      for (int t0 = 0; t0 < K; t0 += kTile) {
        const int nt = min(kTile, K - t0);
        for (int i = tid; i < kTile; i += kQThreads)
          S.hyp[i] = i < nt ? d.hyp[(size_t)l * K + t0 + i] : make_float4(0.f, 0.f, 0.f, -1.f);
        __syncthreads();
        int acc[kTile / 32];
#pragma unroll
        for (int hb = 0; hb < kTile / 32; ++hb) acc[hb] = 0;
#pragma unroll
        for (int hb = 0; hb < kTile / 32; ++hb) {
          if (hb * 32 >= nt) break;  // block-uniform
          const int jn = min(32, nt - hb * 32);
#pragma unroll 4
          for (int j = 0; j < jn; ++j) {
            const float4 e = S.hyp[hb * 32 + j];
            int votes = 0;
#pragma unroll
            for (int k = 0; k < kPPT; ++k) {
              const float du = fsub(pu[k].x, e.x), dv = fsub(pu[k].y, e.y);
              const float d2 = fadd(fmul(du, du), fmul(dv, dv));
              votes += __popc(__ballot_sync(0xffffffffu, mine[k] && (d2 > e.z) && (d2 < e.w)));
            }
            if (lane == j) acc[hb] += votes;
          }
        }
#pragma unroll
        for (int hb = 0; hb < kTile / 32; ++hb) S.cnt[w][hb * 32 + lane] = acc[hb];
        __syncthreads();
        for (int h = tid; h < nt; h += kQThreads) {
          int s = 0;
#pragma unroll
          for (int k = 0; k < kQWarps; ++k) s += S.cnt[k][h];
          if (s) atomicAdd(d.hyp_cnt + (size_t)l * K + t0 + h, s);
        }
        __syncthreads();
      }
    } else {
      // ---- one LS iteration's sums over the chunk (the hypothesis's
      // inliers, fixed over the iterations)
      const double* gst = d.q_st + (size_t)l * 16;
      const bool live = __ldcg(gst + 15) >= 0.0 && __ldcg(gst + 7) != 0.0;
      if (live) {
        const float* sf = d.q_sf + (size_t)l * 16;
        const float cx = __ldcg(sf + 0), cy = __ldcg(sf + 1), cz = __ldcg(sf + 2);
        const float dx = __ldcg(sf + 3), dy = __ldcg(sf + 4), dz = __ldcg(sf + 5);
        const float b1x = __ldcg(sf + 6), b1y = __ldcg(sf + 7), b1z = __ldcg(sf + 8);
        const float b2x = __ldcg(sf + 9), b2y = __ldcg(sf + 10), b2z = __ldcg(sf + 11);
        const float rf = __ldcg(sf + 12);
        const float4 H = __ldcg(d.q_hyp + l);
        for (int k = 0; k < kPPT; ++k) {
          const int sl = c * kPPT + k;  // the slice of the tree
          if (sl >= ns) break;          // block-uniform
          const int i = sl * kQThreads + tid;
          float acc[20];
#pragma unroll
          for (int j = 0; j < 20; ++j) acc[j] = 0.f;
          bool use = i < n;
          float4 qp = make_float4(0.f, 0.f, 0.f, 0.f);
          if (use) {
            const float2 uv = uvs[i];
            const float du = fsub(uv.x, H.x), dv = fsub(uv.y, H.y);
            const float d2 = fadd(fmul(du, du), fmul(dv, dv));
            use = (d2 > H.z) & (d2 < H.w);
            if (use) qp = pts[i];
          }
          const float wx = qp.x - cx, wy = qp.y - cy, wz = qp.z - cz;
          const float wd = wx * dx + wy * dy + wz * dz;
          const float px_ = wx - wd * dx, py_ = wy - wd * dy, pz_ = wz - wd * dz;
          const float rho = sqrtf(px_ * px_ + py_ * py_ + pz_ * pz_);
          if (use && rho > 0.f) {
            const float res = rho - rf;
            const float a1 = (px_ * b1x + py_ * b1y + pz_ * b1z) / rho;
            const float a2 = (px_ * b2x + py_ * b2y + pz_ * b2z) / rho;
            const float J[5] = {-a1, -a2, -wd * a1, -wd * a2, -1.0f};
            int m = 0;
#pragma unroll
            for (int a = 0; a < 5; ++a)
#pragma unroll
              for (int b = a; b < 5; ++b) acc[m++] = J[a] * J[b];
#pragma unroll
            for (int a = 0; a < 5; ++a) acc[15 + a] = J[a] * res;
          }
#pragma unroll
          for (int j = 0; j < 20; ++j) {
            const float v = warp_sum(acc[j]);
            if (lane == 0) red[j][w] = v;
          }
          __syncthreads();
          if (tid < 20) {
            double t = 0.0;
            for (int q2 = 0; q2 < kQWarps; ++q2) t += red[tid][q2];
            d.q_part[(size_t)(s0 + sl) * 20 + tid] = t;
          }
          __syncthreads();
        }
      }
    }
    // ---- arrival; the last chunk's block finishes the phase for the tree
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      s_last = atomicAdd(d.q_done + (size_t)l * kQueuePhases + p, 1) == nc - 1;
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (p == 0) {
        // best hypothesis: most inliers, lowest index on ties
        unsigned long long best = 0ull;
        for (int h = tid; h < K; h += kQThreads) {
          const int cn = __ldcg(d.hyp_cnt + (size_t)l * K + h);
          if (cn > 0) {
            const unsigned long long kk =
                ((unsigned long long)cn << 32) | (unsigned long long)(0xFFFFFFFFu - (uint32_t)h);
            best = kk > best ? kk : best;
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
          best = x > best ? x : best;
        }
        if (lane == 0) sk[w] = best;
        __syncthreads();
        if (tid == 0) {
          for (int k = 1; k < kQWarps; ++k) best = sk[k] > best ? sk[k] : best;
          d.cyl_best[l] = best;
          double* gst = d.q_st + (size_t)l * 16;
          float* gsf = d.q_sf + (size_t)l * 16;
          if (best == 0ull) {
            gst[7] = 0.0;
            gst[15] = -1.0;  // no hypothesis with inliers: the vertex-line model stays
          } else {
            const int h = (int)(0xFFFFFFFFu - (uint32_t)(best & 0xffffffffull));
            const CylD cy = d.cyl_all[l];
            const CylFrame f = make_frame(d, cy);
            const float4 e = d.hyp[(size_t)l * K + h];
            st[0] = f.ox + (double)e.x * f.e1x + (double)e.y * f.e2x;
            st[1] = f.oy + (double)e.x * f.e1y + (double)e.y * f.e2y;
            st[2] = f.oz + (double)e.x * f.e1z + (double)e.y * f.e2z;
            const double an =
                sqrt((double)f.ax * f.ax + (double)f.ay * f.ay + (double)f.az * f.az);
            st[3] = f.ax / an; st[4] = f.ay / an; st[5] = f.az / an;
            // the hypothesis radius: sqrt(hi2) - tau reproduces the circle's r
            const Hyp Hh = make_hyp(kp, h, cy.id, n, [&](uint32_t i) { return uvs[i]; });
            st[6] = Hh.r;
            st[7] = 1.0;
            st[14] = (double)(int)(best >> 32);
            st[15] = (double)h;
            float sfl[13];
            ls_frame(st, sfl);
            for (int j = 0; j < 16; ++j) gst[j] = st[j];
            for (int j = 0; j < 13; ++j) gsf[j] = sfl[j];
            d.q_hyp[l] = e;
            if (P == 1) queue_write_cylinder(d, l, st, (int)(best >> 32));
          }
        }
      } else {
        if (tid == 0)
          for (int j = 0; j < 16; ++j) st[j] = __ldcg(d.q_st + (size_t)l * 16 + j);
        __syncthreads();
        const bool has_model = st[15] >= 0.0;
        if (has_model && st[7] != 0.0 && w == 0) {
          if (lane < 20) {
            double t = 0.0;
            for (int k = 0; k < ns; ++k) t += __ldcg(d.q_part + (size_t)(s0 + k) * 20 + lane);
            ssum[lane] = t;
          }
          __syncwarp();
          const bool solved = warp_chol_solve<5>(ssum, ssum + 15, sxls);
          __syncwarp();
          if (lane == 0) {
            if (solved) {
              const double* x = sxls;
              const d3 cc = mk3(st[0], st[1], st[2]), dd = mk3(st[3], st[4], st[5]);
              const d3 b1 = mk3(st[8], st[9], st[10]), b2 = mk3(st[11], st[12], st[13]);
              d3 c2 = add3(add3(cc, scl3(x[0], b1)), scl3(x[1], b2));
              d3 d2 = add3(add3(dd, scl3(x[2], b1)), scl3(x[3], b2));
              d2 = scl3(1.0 / norm3(d2), d2);
              st[0] = c2.x; st[1] = c2.y; st[2] = c2.z;
              st[3] = d2.x; st[4] = d2.y; st[5] = d2.z;
              st[6] = st[6] + x[4];
              float sfl[13];
              ls_frame(st, sfl);
              float* gsf = d.q_sf + (size_t)l * 16;
              for (int j = 0; j < 13; ++j) gsf[j] = sfl[j];
            } else {
              st[7] = 0.0;
            }
            double* gst = d.q_st + (size_t)l * 16;
            for (int j = 0; j < 16; ++j) gst[j] = st[j];
          }
        }
        __syncthreads();
        if (tid == 0 && has_model && p == P - 1) queue_write_cylinder(d, l, st, (int)st[14]);
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

template <int kPPT, int kTile>
void set_queue_attr() {
  cudaFuncSetAttribute(k_cyl_queue<kPPT, kTile>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(QueueSmem<kTile>));
}

template <int kPPT, int kTile>
void launch_queue_t(const Dev& d, const KParams& kp, int blocks, cudaStream_t st) {
  k_cyl_queue<kPPT, kTile><<<blocks, kQThreads, sizeof(QueueSmem<kTile>), st>>>(d, kp);
}

template <int kPPT>
bool launch_queue_tile(const Dev& d, const KParams& kp, int tile, int blocks, cudaStream_t st) {
  switch (tile) {
    case 64: launch_queue_t<kPPT, 64>(d, kp, blocks, st); return true;
    case 128: launch_queue_t<kPPT, 128>(d, kp, blocks, st); return true;
    case 256: launch_queue_t<kPPT, 256>(d, kp, blocks, st); return true;
    case 512: launch_queue_t<kPPT, 512>(d, kp, blocks, st); return true;
    case 1024: launch_queue_t<kPPT, 1024>(d, kp, blocks, st); return true;
  }
  return false;
}

template <int kPPT>
void set_queue_attrs() {
  set_queue_attr<kPPT, 64>();
  set_queue_attr<kPPT, 128>();
  set_queue_attr<kPPT, 256>();
  set_queue_attr<kPPT, 512>();
  set_queue_attr<kPPT, 1024>();
}

}  // namespace

void init_queue_attributes() {
  set_queue_attrs<1>();
  set_queue_attrs<2>();
  set_queue_attrs<4>();
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
  const int chunk = kp.q_chunk, tile = kp.q_tile;
  k_cyl_queue_prep<<<1, 1024, 0, st>>>(d, kp, only, chunk);
  const int blocks = kp.q_blocks;
  bool ok = false;
  if (chunk == 256) ok = launch_queue_tile<1>(d, kp, tile, blocks, st);
  else if (chunk == 512) ok = launch_queue_tile<2>(d, kp, tile, blocks, st);
  else if (chunk == 1024) ok = launch_queue_tile<4>(d, kp, tile, blocks, st);
  return ok ? 2 : 1;
}

}  // namespace sg
