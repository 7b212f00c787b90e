// context.cu — the C ABI (include/sloam_gb300.h): context life cycle, the
// device arena, host<->device staging, the exact boundary tables, CUDA-graph
// capture of the keyframe pipeline, and the stage entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "proposal.cuh"

using namespace sg;

// ------------------------------------------------------------- parameters
extern "C" void sloam_params_default(sloam_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->scans_per_sweep = 1;
  p->min_tree_models = 5;
  p->min_ground_models = 36;
  p->max_lidar_dist = 20.0;
  p->max_ground_lidar_dist = 25.0;
  p->min_ground_lidar_dist = 5.0;
  p->two_step_optim = 1;
  p->ground_radii_bins = 2;
  p->ground_theta_bins = 18;
  p->ground_retain_thresh = 0.05;
  p->ground_match_thresh = 1.0;
  p->rough_tree_match_thresh = 2.5;
  p->tree_match_thresh = 0.5;
  p->max_tree_radius = 0.3;
  p->max_axis_theta = 10.0;
  p->max_focus_outlier_distance = 0.5;
  p->add_new_tree_thresh_dist = 1.5;
  p->features_per_tree = 20;
  p->num_ground_features = 5;
  p->default_tree_radius = 0.2;
  p->min_planes = 0.1 * 2 * 18;
  p->beam_cluster_threshold = 0.5f;
  p->max_dist_to_centroid = 0.2f;
  p->min_vertex_size = 4;
  p->min_landmark_size = 5;
  p->min_landmark_height = 1.0f;
  p->fov_up_deg = 22.5f;
  p->fov_down_deg = -22.5f;
  p->img_w = 2048;
  p->img_h = 64;
  p->do_destagger = 1;
  p->cc_dist_threshold = 1.0f;
  p->trellis_min_cluster = 80;
  p->trellis_min_beam_points = 3;
  p->trellis_min_vertices = 16;
  p->trellis_max_vertices = 56;
  p->line_ransac_thresh = 0.25;
  p->line_ransac_max_iter = 50;
  p->line_ransac_probability = 0.99;
  p->min_tree_height_sq = 1.5;
  p->root_plane_max_dist = 2.0;
  p->plane_match_thresh = 1.0;
  p->huber_delta = 0.1;
  p->seed = 0;
  p->cyl_mode = 0;
  p->cyl_hypotheses = 256;
  p->cyl_inlier_thresh = 0.03f;
  p->cyl_ls_iters = 3;
  p->cyl_max_hyp_radius = 1.0f;
  p->gn_iters = 10;
  p->max_landmarks = 1024;
  p->max_map = 4096;
  p->max_ground = 0;
  p->batch_slots = 8;
  p->prop_samples = 8;
  p->prop_min_inlier_ratio = 0.6f;
  p->pose_solver = 0;
  p->lm_max_iters = 50;
  p->cyl_chunk_points = 256;
  p->cyl_hyp_tile = 256;
  p->cyl_queue_blocks = 0;
}

// sizeof() of every ABI struct, for binding checks.
extern "C" int sloam_abi_sizes(int32_t* out, int n) {
  const int32_t s[] = {(int32_t)sizeof(sloam_params), (int32_t)sizeof(sloam_se3),
                       (int32_t)sizeof(sloam_landmarks), (int32_t)sizeof(sloam_cylinder),
                       (int32_t)sizeof(sloam_plane), (int32_t)sizeof(sloam_scan_out),
                       (int32_t)sizeof(sloam_models_out), (int32_t)sizeof(sloam_run_out)};
  const int k = (int)(sizeof(s) / sizeof(s[0]));
  for (int i = 0; i < k && i < n; ++i) out[i] = s[i];
  return k;
}

namespace sg {

// ------------------------------------------------------ boundary tables
namespace {
int32_t f2o(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? -(int32_t)(u & 0x7fffffffu) : (int32_t)u;
}
float o2f(int32_t o) {
  uint32_t u = o < 0 ? (0x80000000u | (uint32_t)(-o)) : (uint32_t)o;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
// smallest float v in [lo, hi] with g(v) >= k (g non-decreasing); hi if none
template <typename G>
float first_at_least(G g, int k, float lo, float hi) {
  int64_t a = f2o(lo), b = f2o(hi);  // 64-bit: the span exceeds INT32_MAX
  if (g(o2f((int32_t)a)) >= k) return o2f((int32_t)a);
  if (g(o2f((int32_t)b)) < k) return o2f((int32_t)b);
  while (b - a > 1) {
    const int64_t m = a + (b - a) / 2;
    if (g(o2f((int32_t)m)) >= k) b = m;
    else a = m;
  }
  return o2f((int32_t)b);
}
inline float ref_min(float a, float b) { return (b < a) ? b : a; }
inline float ref_max(float a, float b) { return (a < b) ? b : a; }
}  // namespace

// Column of a float yaw exactly as inference.cpp:111-121 computes it.
void build_px_table(const sloam_params& p, float* tab) {
  const int W = p.img_w;
  auto col = [W](float yaw) {
    float proj_x = 0.5 * (yaw / M_PI + 1.0);
    proj_x *= W;
    proj_x = std::floor(proj_x);
    proj_x = ref_min(W - 1.0f, proj_x);
    proj_x = ref_max(0.0f, proj_x);
    return (int)proj_x;
  };
  tab[0] = -INFINITY;
  for (int k = 1; k < W; ++k) tab[k] = first_at_least(col, k, -4.0f, 4.0f);
  tab[W] = INFINITY;
}

// Row of a point exactly as inference.cpp:108-126 computes it, as a table on
// q = z / range itself (the float division the reference computes):
// pitch = asinf(q) correctly rounded (the projection's contract, the float
// of the FP64 asin), then the row in float arithmetic, unfused.  The row falls
// as q grows, so the table holds tab[k] = smallest float q in [-1, 1] whose
// row is <= H-1-k (k = 1..H-1; +inf when no q reaches it): the row of q is
// H-1 minus the number of k with q >= tab[k].  A q outside [-1, 1] (or NaN)
// has a NaN pitch, which the reference's clamps send to row H-1.
void build_line_k_table(const sloam_params& p, double* tab) {
  const double log_p = std::log(1.0 - p.line_ransac_probability);
  const double eps = std::numeric_limits<double>::epsilon();
  for (int V = 0; V <= kLineKMax; ++V)
    for (int c = 0; c <= kLineKMax; ++c) {
      double k = 1.0;
      if (V > 0 && c > 0 && c <= V) {
        const double w = (double)c / V;
        double p_no = 1.0 - w * w;
        p_no = std::max(eps, std::min(1.0 - eps, p_no));
        k = log_p / std::log(p_no);
      }
      tab[V * (kLineKMax + 1) + c] = k;
    }
}

void build_py_table(const sloam_params& p, float* tab) {
  const int H = p.img_h;
  const KParams kp = make_kparams(p);
  const float fd = kp.fov_down_abs, fov = kp.fov;
  auto g = [H, fd, fov](float q) {
    const float pitch = (float)std::asin((double)q);
    float t = (pitch + fd) / fov;
    float y = (1.0f - t) * (float)H;
    y = std::floor(y);
    y = ref_min(H - 1.0f, y);
    y = ref_max(0.0f, y);
    return H - 1 - (int)y;
  };
  tab[0] = -INFINITY;
  for (int k = 1; k < H; ++k)
    tab[k] = g(1.0f) >= k ? first_at_least(g, k, -1.0f, 1.0f) : INFINITY;
  tab[H] = INFINITY;
}

// Theta and radius bins of sloam.cpp:346-357 as float boundary tables, and
// the float window equivalent to r < maxG && r > minG in double.
void build_ground_tables(const sloam_params& p, float* tb, float* rb, float* r_lo, float* r_hi) {
  const int Rb = p.ground_radii_bins, Tb = p.ground_theta_bins;
  const double maxG = p.max_ground_lidar_dist, minG = p.min_ground_lidar_dist;
  auto tbin = [Tb](float th) {
    int t = (int)std::floor((kPIDEF + (double)th) / (2 * kPIDEF / (double)Tb));
    return std::max(0, std::min(t, Tb - 1));
  };
  auto rbin = [Rb, maxG](float r) {
    int t = (int)std::floor((double)r / (maxG / (double)Rb));
    return std::max(0, std::min(t, Rb - 1));
  };
  tb[0] = -INFINITY;
  for (int k = 1; k < Tb; ++k) tb[k] = first_at_least(tbin, k, -4.0f, 4.0f);
  tb[Tb] = INFINITY;
  rb[0] = -INFINITY;
  const float rmax = (float)maxG * 2.0f + 1.0f;
  for (int k = 1; k < Rb; ++k) rb[k] = first_at_least(rbin, k, 0.0f, rmax);
  rb[Rb] = INFINITY;
  // r < maxG (double) <=> r <= hi ; r > minG <=> r >= lo
  float hi = (float)maxG;
  while ((double)hi >= maxG) hi = std::nextafter(hi, -INFINITY);
  while ((double)std::nextafter(hi, INFINITY) < maxG) hi = std::nextafter(hi, INFINITY);
  float lo = (float)minG;
  while ((double)lo <= minG) lo = std::nextafter(lo, INFINITY);
  while ((double)std::nextafter(lo, -INFINITY) > minG) lo = std::nextafter(lo, -INFINITY);
  *r_lo = lo;
  *r_hi = hi;
}

}  // namespace sg

// Test hook (not part of the public header): the host-built boundary tables
// a context would upload.  px_tab [img_w+1], tb [theta_bins+1],
// rb [radii_bins+1], lohi [2], py_tab [img_h+1].
extern "C" int sloam_internal_tables(const sloam_params* p, float* px_tab, float* tb, float* rb,
                                     float* lohi, float* py_tab) {
  if (!p) return SLOAM_ERR_ARG;
  sg::build_px_table(*p, px_tab);
  sg::build_py_table(*p, py_tab);
  sg::build_ground_tables(*p, tb, rb, lohi, lohi + 1);
  return SLOAM_OK;
}

// ================================================================ context
// Keyframes per batch projection launch: 64 when the scans are already in
// device memory (one launch group for a 64-keyframe batch: the grid's ramp
// and tail are paid once; measured 30 us per 16 keyframes against 37 us in
// chunks of 16), 4 when they stream from host memory (uploads of the next
// chunk overlap the projection of this one and the keyframes of the last;
// the first keyframes start after 9 MB of upload: the host batch ran 1.3 %
// faster than in chunks of 8, and 2 and 16 were slower).
// Consecutive chunks alternate between two scratch sets, so a chunk's label
// kernels overlap the next chunk's projection.
constexpr int kFrontChunkHost = 4, kFrontChunkDevice = 64;
constexpr int kFrontChunkMax = kFrontChunkDevice;

// A slot's second stream and the two events of the fork and join inside
// its keyframe graph.
struct Fork {
  cudaStream_t aux = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
bool create_fork(Fork& f) {
  if (!f.aux && cudaStreamCreateWithFlags(&f.aux, cudaStreamNonBlocking) != cudaSuccess) return false;
  if (!f.fork && cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming) != cudaSuccess) return false;
  if (!f.join && cudaEventCreateWithFlags(&f.join, cudaEventDisableTiming) != cudaSuccess) return false;
  return true;
}
void destroy_fork(Fork& f) {
  if (f.aux) {
    cudaStreamSynchronize(f.aux);
    cudaStreamDestroy(f.aux);
  }
  if (f.fork) cudaEventDestroy(f.fork);
  if (f.join) cudaEventDestroy(f.join);
  f = Fork{};
}

// Captured keyframe graphs of one slot, keyed
// [first scan][point labels][state update][projection done by a batch launch].
struct GraphSet {
  cudaGraphExec_t g[2][2][2][2] = {};
  int launches[2][2][2][2] = {};
};

struct sloam_ctx {
  sloam_params P;
  KParams kp;
  int device = 0;
  cudaStream_t st = nullptr;
  Dev d{};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  // pinned staging
  Counters* h_cnt = nullptr;
  double* h_pose = nullptr;     // 21 doubles
  InPtrs* h_in = nullptr;       // per-keyframe input pointer blocks (batch)
  double* h_poses = nullptr;    // per-keyframe estimates (batch)
  int h_batch_cap = 0;
  // their device copies, one upload per batch (each slot takes its
  // keyframe's block with a kernel, not a host copy: a small copy would
  // queue behind the batch's scan uploads on the copy engine)
  InPtrs* d_in_all = nullptr;
  double* d_poses_all = nullptr;
  int d_batch_cap = 0;
  bool first_scan = true;
  std::string err;
  int64_t launches = 0;
  int64_t last_launches = 0;
  GraphSet gx;
  int cc_iter_limit = -1;  // sloam_set_cc_iter_limit override (-1: the default)
  // further keyframe slots of a batch (slot 0 is the fields above)
  struct Slot {
    Dev d{};
    void* arena = nullptr;
    size_t arena_bytes = 0;
    cudaStream_t st = nullptr;
    GraphSet gx;
    cudaEvent_t ev = nullptr;
    Fork fk;
  };
  std::vector<Slot> extra;
  cudaEvent_t ev_main = nullptr;
  Fork fk;  // the context's own keyframe graph
  // batch projection: a1-a2 of a whole batch on its own stream, one launch
  // per kernel and chunk of keyframes, into per-keyframe buffers
  // fe_st: the projection kernel of each chunk; fe_st2: the chunk's label
  // and compaction kernels, so the next chunk's projection overlaps them
  // (the chunk scratch alternates between two sets); fe_cp: the scan uploads
  // of the host entry point, back to back, each chunk's projection waiting
  // for its own chunk's copies only
  cudaStream_t fe_st = nullptr, fe_st2 = nullptr, fe_cp = nullptr;
  void* fb = nullptr;            // [fb_cap] per-keyframe projection buffers
  size_t fb_stride = 0;          // bytes per keyframe
  int32_t* fb_pix = nullptr;     // [2][kFrontChunkMax * N] point pixels of the chunks in flight
  unsigned long long* fb_pkey = nullptr;  // [2][kFrontChunkMax * N] pixel keys, kept all-ones
  int fe_chunk = kFrontChunkHost;         // keyframes per projection launch of this batch
  int fb_cap = 0;
  bool fb_upload = false;        // the buffers include scan upload space
  FrontRef* d_refs = nullptr;    // [fb_cap]
  FrontRef* h_refs = nullptr;    // [fb_cap], pinned
  int32_t* fb_fe = nullptr;      // [fb_cap * 4] projection counters
  // chunk c: [3c] before its projection, [3c+1] after it, [3c+2] after
  // its label and compaction kernels
  std::vector<cudaEvent_t> ev_fe;
  std::vector<cudaEvent_t> ev_cp;  // [chunk] the chunk's uploads done
  int fe_chunks = 0, fe_nkf = 0;
  // learned proposal: bf16 network weights in the tensor-core layout
  unsigned char* prop_tc = nullptr;
  // host batch staging
  int32_t* d_out_i = nullptr;   // [2 * cap] success, ncyl
  double* d_out_pose = nullptr; // [7 * cap]
  int out_cap = 0;
};

namespace {

int fail(sloam_ctx* c, int code, const char* what, cudaError_t e = cudaSuccess) {
  if (c) {
    char buf[512];
    if (e != cudaSuccess)
      std::snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorName(e),
                    cudaGetErrorString(e));
    else
      std::snprintf(buf, sizeof(buf), "%s", what);
    c->err = buf;
  }
  return code;
}

#define CK(call)                                                  \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return fail(ctx, SLOAM_ERR_CUDA, #call, e_); \
  } while (0)

struct Carver {
  char* base;
  size_t off = 0;
  bool dry;
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~(size_t)255;
    T* p = dry ? nullptr : reinterpret_cast<T*>(base + off);
    off += sizeof(T) * std::max<size_t>(n, 1);
    return p;
  }
};

void carve(Dev& d, Carver& c, int n_blk) {
  const int N = d.N;
  d.in = c.take<InPtrs>(1);
  d.buf_xyzi = c.take<float4>(N);
  d.buf_plabel = c.take<uint8_t>(N);
  d.buf_mask_in = c.take<uint8_t>(N);
  d.pix = c.take<int32_t>(N);
  d.pkey = c.take<unsigned long long>(N);
  d.range_img = c.take<float>(N);
  d.mask = c.take<uint8_t>(N);
  d.tree = c.take<float4>(N);
  d.gbits = c.take<uint32_t>((size_t)((N + 1023) / 1024) * 32 + 32);
  d.blk = c.take<int32_t>(n_blk);
  d.ground_idx = c.take<int32_t>(N);
  d.ground = c.take<float4>(d.cap_ground);
  d.px_tab = c.take<float>(d.W + 1);
  d.line_k = c.take<double>((size_t)(kLineKMax + 1) * (kLineKMax + 1));
  d.py_tab = c.take<float>(d.H + 1);
  d.tb_tab = c.take<float>(4096);
  d.rb_tab = c.take<float>(4096);
  d.parent = c.take<uint32_t>(N);
  d.label = c.take<uint32_t>(N);
  d.rank = c.take<uint32_t>(std::max(N, 4 * d.cap_cand));
  d.comp_size = c.take<int32_t>(N);
  d.comp_cmin = c.take<int32_t>(N);
  d.comp_cmax = c.take<int32_t>(N);
  d.comp_cand = c.take<int32_t>(N);
  d.cand_comp = c.take<int32_t>(d.cap_cand);
  d.rc = c.take<int32_t>((size_t)d.cap_cand * d.H);
  d.roff = c.take<int32_t>((size_t)d.cap_cand * d.H + 1);
  d.bucket = c.take<int32_t>(N);
  d.wide_list = c.take<int32_t>((size_t)d.cap_cand * d.H);
  d.kept = c.take<float4>(N);
  d.vmed = c.take<float4>((size_t)d.cap_cand * d.H);
  d.vrad = c.take<double>((size_t)d.cap_cand * d.H);
  d.vkept = c.take<int32_t>((size_t)d.cap_cand * d.H);
  d.cand_nv = c.take<int32_t>(d.cap_cand);
  d.cand_lm = c.take<int32_t>(d.cap_cand);
  d.lm_tree = c.take<int32_t>(d.cap_lm);
  d.lm_vbeg = c.take<int32_t>(d.cap_lm + 1);
  d.lm_vxyz = c.take<float>((size_t)d.cap_v * 3);
  d.lm_vrad = c.take<double>(d.cap_v);
  d.lm_vrow = c.take<int32_t>(d.cap_v);
  d.lm_pbeg = c.take<int32_t>(d.cap_v + 1);
  d.lm_pts = c.take<float4>(d.cap_p);
  d.lm_cbeg = c.take<int32_t>(d.cap_lm + 1);
  d.lm_cpts = c.take<float4>(d.cap_cluster);
  d.lm_vsrc = c.take<int32_t>(d.cap_v);
  d.bin_of = c.take<int32_t>(d.cap_ground);
  d.bin_cnt = c.take<int32_t>(d.n_bins);
  d.bin_off = c.take<int32_t>(d.n_bins + 1);
  d.bin_keys = c.take<unsigned long long>(d.cap_ground);
  d.plane_all = c.take<PlaneD>(d.n_bins);
  d.plane_feat_all = c.take<float4>((size_t)d.n_bins * d.G);
  d.planes = c.take<PlaneD>(d.n_bins);
  d.plane_feat = c.take<float4>((size_t)d.n_bins * d.G);
  d.prev_planes = c.take<PlaneD>(d.n_bins);
  d.prev_feat = c.take<float4>((size_t)d.n_bins * d.G);
  d.cyl_all = c.take<CylD>(d.cap_lm);
  d.cyl_feat_all = c.take<float4>((size_t)d.cap_lm * d.F);
  d.cyl_best = c.take<unsigned long long>(d.cap_lm);
  d.cyls = c.take<CylD>(d.cap_lm);
  d.cyl_feat = c.take<float4>((size_t)d.cap_lm * d.F);
  d.buf_map = c.take<sloam_cylinder>(d.cap_map);
  d.cyl_match = c.take<int32_t>(d.cap_lm);
  d.plane_match = c.take<int32_t>(d.n_bins);
  d.match_out = c.take<int32_t>(d.cap_lm);
  d.map_pts = c.take<double>((size_t)d.cap_map * 9);
  d.map_f = c.take<float4>((size_t)d.cap_map * 3);
  d.res_tab = c.take<float>(((size_t)d.cap_lm * d.F + (size_t)d.n_bins * d.G) * 12);
  d.lm_uv = c.take<float2>((size_t)d.cap_cluster + d.cap_p);  // cluster | vertex points
  d.hyp = c.take<float4>((size_t)d.cap_lm * std::max(d.K, 1));
  d.hyp_cnt = c.take<int32_t>((size_t)d.cap_lm * std::max(d.K, 1));
  d.qctl = c.take<QueueCtl>(1);
  d.q_order = c.take<int32_t>(d.cap_lm);
  d.q_off = c.take<int32_t>((size_t)d.cap_lm + 1);
  d.q_soff = c.take<int32_t>((size_t)d.cap_lm + 1);
  d.q_ready = c.take<int32_t>(d.cap_lm);
  d.q_done = c.take<int32_t>((size_t)d.cap_lm * kQueuePhases);
  d.q_st = c.take<double>((size_t)d.cap_lm * 16);
  d.q_sf = c.take<float>((size_t)d.cap_lm * 16);
  d.q_hyp = c.take<float4>(d.cap_lm);
  // 1024-point LS slices, at most one partial slice per tree
  d.q_cap_chunks = (int)(((size_t)d.cap_cluster + d.cap_p) / 1024 + d.cap_lm);
  d.q_part = c.take<float>((size_t)d.q_cap_chunks * 20);
  const size_t ps = (size_t)std::max(d.prop_cap, 1);
  d.prop_x = c.take<float>(ps * 384);
  d.prop_f = c.take<float4>(ps);
  d.prop_out = c.take<float>(ps * 8);
  d.pflag = c.take<int32_t>(d.cap_lm);
  d.pose_io = c.take<double>(32);
  d.cnt = c.take<Counters>(1);
  d.prop_err = c.dry ? nullptr : &d.cnt->prop_err;
}

int check_params(const sloam_params& p) {
  // pixel keys carry a 24-bit point index
  if (p.img_w < 32 || p.img_h < 1 || (int64_t)p.img_w * p.img_h > (1 << 24)) return 1;
  if (p.ground_radii_bins < 1 || p.ground_theta_bins < 1 ||
      p.ground_radii_bins * p.ground_theta_bins > 4096)
    return 1;
  if (p.features_per_tree < 0 || p.num_ground_features < 0) return 1;
  if (p.trellis_max_vertices < 1 || p.trellis_max_vertices > 4096) return 1;
  if (p.cyl_hypotheses < 0 || p.cyl_hypotheses > 4096 || p.line_ransac_max_iter > 256) return 1;
  if (!(p.ground_retain_thresh > 0)) return 1;
  if (p.batch_slots < 0 || p.batch_slots > 64) return 1;
  if (p.cyl_mode < 0 || p.cyl_mode > 2 || p.prop_samples < 1 || p.prop_samples > 8) return 1;
  if (p.pose_solver < 0 || p.pose_solver > 1 || p.lm_max_iters < 1 || p.lm_max_iters > 1000)
    return 1;
  if (p.cyl_ls_iters < 0 || p.cyl_ls_iters > kQueuePhases - 1 || p.max_landmarks > 4096)
    return 1;
  if (!queue_shape_valid(p.cyl_chunk_points, p.cyl_hyp_tile) || p.cyl_queue_blocks < 0 ||
      p.cyl_queue_blocks > 65536)
    return 1;
  return 0;
}

void destroy_graphs(GraphSet& gs) {
  for (auto& a : gs.g)
    for (auto& b : a)
      for (auto& c : b)
        for (auto& g : c)
          if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
          }
}

// Sizes, carves and initialises one slot's device state.
int init_dev(sloam_ctx* ctx, const sloam_params& P, Dev& d, void*& arena, size_t& arena_bytes,
             cudaStream_t st) {
  d.H = P.img_h;
  d.W = P.img_w;
  d.N = P.img_h * P.img_w;
  d.cap_ground = P.max_ground > 0 ? std::min(P.max_ground, d.N) : d.N;
  d.cap_cand = d.N / (std::max(P.trellis_min_cluster, 0) + 1) + 1;
  d.cap_lm = std::max(1, std::min(P.max_landmarks, d.cap_cand));
  d.cap_v = d.cap_lm * P.trellis_max_vertices;
  d.cap_p = d.N;
  d.cap_cluster = d.N;
  d.cap_map = std::max(1, P.max_map);
  d.n_bins = P.ground_radii_bins * P.ground_theta_bins;
  d.F = P.features_per_tree;
  d.G = P.num_ground_features;
  d.K = P.cyl_hypotheses;
  d.prop_cap = P.cyl_mode == 2 ? d.cap_lm * P.prop_samples : 0;
  d.prop_tc = ctx->prop_tc;
  const int n_blk = d.N / 256 + 64;
  Carver dry{nullptr, 0, true};
  carve(d, dry, n_blk);
  const size_t bytes = dry.off + 256;
  if (arena && bytes > arena_bytes) {
    cudaFree(arena);
    arena = nullptr;
  }
  if (!arena) {
    CK(cudaMalloc(&arena, bytes));
    arena_bytes = bytes;
  }
  Carver real{reinterpret_cast<char*>(arena), 0, false};
  carve(d, real, n_blk);
  // tables
  std::vector<float> tab(d.W + 1), ptab(d.H + 1), tb(4096), rb(4096);
  build_px_table(P, tab.data());
  build_py_table(P, ptab.data());
  build_ground_tables(P, tb.data(), rb.data(), &d.r_lo, &d.r_hi);
  std::vector<double> lk((size_t)(kLineKMax + 1) * (kLineKMax + 1));
  build_line_k_table(P, lk.data());
  CK(cudaMemcpyAsync(d.line_k, lk.data(), sizeof(double) * lk.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.px_tab, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.py_tab, ptab.data(), sizeof(float) * ptab.size(), cudaMemcpyHostToDevice,
                     st));
  CK(cudaMemcpyAsync(d.tb_tab, tb.data(), sizeof(float) * (P.ground_theta_bins + 1),
                     cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.rb_tab, rb.data(), sizeof(float) * (P.ground_radii_bins + 1),
                     cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(d.pkey, 0xFF, sizeof(unsigned long long) * d.N, st));
  CK(cudaMemsetAsync(d.cnt, 0, sizeof(Counters), st));
  CK(cudaMemsetAsync(d.in, 0, sizeof(InPtrs), st));
  CK(cudaStreamSynchronize(st));
  return SLOAM_OK;
}

void free_front(sloam_ctx* ctx);

int setup(sloam_ctx* ctx, const sloam_params& P) {
  free_front(ctx);  // sized by the scan and ground capacities
  ctx->P = P;
  ctx->kp = make_kparams(P);
  if (ctx->cc_iter_limit >= 0) ctx->kp.cc_iter_limit = ctx->cc_iter_limit;
  int st = init_dev(ctx, P, ctx->d, ctx->arena, ctx->arena_bytes, ctx->st);
  if (st) return st;
  destroy_graphs(ctx->gx);
  const int ns = std::max(1, std::min(P.batch_slots, 64)) - 1;
  while ((int)ctx->extra.size() > ns) {
    auto& s = ctx->extra.back();
    cudaStreamSynchronize(s.st);
    destroy_graphs(s.gx);
    if (s.arena) cudaFree(s.arena);
    if (s.ev) cudaEventDestroy(s.ev);
    if (s.st) cudaStreamDestroy(s.st);
    destroy_fork(s.fk);
    ctx->extra.pop_back();
  }
  ctx->extra.resize(ns);
  if (!create_fork(ctx->fk)) return fail(ctx, SLOAM_ERR_CUDA, "aux stream of the context");
  for (auto& s : ctx->extra) {
    if (!s.st) CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    if (!s.ev) CK(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming));
    if (!create_fork(s.fk)) return fail(ctx, SLOAM_ERR_CUDA, "aux stream of a slot");
    destroy_graphs(s.gx);
    if ((st = init_dev(ctx, P, s.d, s.arena, s.arena_bytes, s.st))) return st;
  }
  if (!ctx->ev_main) CK(cudaEventCreateWithFlags(&ctx->ev_main, cudaEventDisableTiming));
  ctx->first_scan = true;
  return SLOAM_OK;
}

// Reads back counters and pose; maps overflow / device errors to a status.
int sync_counters(sloam_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_cnt, ctx->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(ctx->h_pose, ctx->d.pose_io, sizeof(double) * 21, cudaMemcpyDeviceToHost,
                     ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  CK(cudaGetLastError());
  if (ctx->h_cnt->overflow)
    return fail(ctx, SLOAM_ERR_CAPACITY, "a context capacity was exceeded (overflow flags set)");
  if (ctx->h_cnt->cc_iter_exceeded)
    return fail(ctx, SLOAM_ERR_TIMEOUT, "connected-components union loop hit its iteration limit");
  if (ctx->h_cnt->prop_err)
    return fail(ctx, SLOAM_ERR_TIMEOUT, "proposal network: a tensor-core wait gave up");
  if (ctx->h_cnt->queue_err)
    return fail(ctx, SLOAM_ERR_TIMEOUT, "cylinder work queue: a wait for a tree's phase gave up");
  return SLOAM_OK;
}

// cyl_mode 2 runs the proposal network: its weights must be loaded
int need_weights(sloam_ctx* ctx) {
  if (ctx->P.cyl_mode == 2 && !ctx->prop_tc)
    return fail(ctx, SLOAM_ERR_ARG, "cyl_mode 2 needs sloam_set_proposal_weights first");
  return SLOAM_OK;
}

int set_inputs(sloam_ctx* ctx, const float4* xyzi, const uint8_t* pl, const uint8_t* mi,
               const sloam_cylinder* map, int n_map) {
  InPtrs& h = ctx->h_in[0];
  h.xyzi = xyzi;
  h.plabel = pl;
  h.mask_in = mi;
  h.map = map;
  h.tree = ctx->d.tree;
  h.ground = ctx->d.ground;
  h.fe = nullptr;
  h.tflag = nullptr;
  h.gidx = nullptr;
  h.n_map = n_map;
  h.destag = 0;
  CK(cudaMemcpyAsync(ctx->d.in, &h, sizeof(InPtrs), cudaMemcpyHostToDevice, ctx->st));
  // the pinned block must stay unchanged until the copy ran
  CK(cudaStreamSynchronize(ctx->st));
  return SLOAM_OK;
}

int upload_pose(sloam_ctx* ctx, const sloam_se3* pose) {
  for (int j = 0; j < 4; ++j) ctx->h_pose[j] = pose->q[j];
  for (int j = 0; j < 3; ++j) ctx->h_pose[4 + j] = pose->t[j];
  CK(cudaMemcpyAsync(ctx->d.pose_io, ctx->h_pose, sizeof(double) * 7, cudaMemcpyHostToDevice,
                     ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return SLOAM_OK;
}

int upload_landmarks(sloam_ctx* ctx, const sloam_landmarks* lm, int* nl, int* nv, int* np,
                     int* ncl) {
  Dev& d = ctx->d;
  *nl = lm ? lm->n_landmarks : 0;
  *nv = *nl ? lm->vertex_begin[*nl] : 0;
  *np = *nv ? lm->point_begin[*nv] : 0;
  *ncl = 0;
  if (*nl > d.cap_lm || *nv > d.cap_v || *np > d.cap_p)
    return fail(ctx, SLOAM_ERR_CAPACITY, "landmarks exceed the context capacity");
  if (*nl == 0) {
    const int zero = 0;
    CK(cudaMemcpyAsync(d.lm_vbeg, &zero, 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d.lm_cbeg, &zero, 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SLOAM_OK;
  }
  CK(cudaMemcpyAsync(d.lm_tree, lm->tree_id, 4 * *nl, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(d.lm_vbeg, lm->vertex_begin, 4 * (*nl + 1), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(d.lm_vxyz, lm->vertex_xyz, 12 * (size_t)*nv, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(d.lm_vrad, lm->vertex_radius, 8 * (size_t)*nv, cudaMemcpyHostToDevice,
                     ctx->st));
  if (lm->vertex_row)
    CK(cudaMemcpyAsync(d.lm_vrow, lm->vertex_row, 4 * (size_t)*nv, cudaMemcpyHostToDevice,
                       ctx->st));
  CK(cudaMemcpyAsync(d.lm_pbeg, lm->point_begin, 4 * (size_t)(*nv + 1), cudaMemcpyHostToDevice,
                     ctx->st));
  if (*np)
    CK(cudaMemcpyAsync(d.lm_pts, lm->point_xyzi, 16 * (size_t)*np, cudaMemcpyHostToDevice,
                       ctx->st));
  std::vector<int32_t> zeros;
  if (lm->cluster_begin && lm->cluster_xyzi) {
    *ncl = lm->cluster_begin[*nl];
    if (*ncl > d.cap_cluster) return fail(ctx, SLOAM_ERR_CAPACITY, "cluster points exceed capacity");
    CK(cudaMemcpyAsync(d.lm_cbeg, lm->cluster_begin, 4 * (*nl + 1), cudaMemcpyHostToDevice,
                       ctx->st));
    if (*ncl)
      CK(cudaMemcpyAsync(d.lm_cpts, lm->cluster_xyzi, 16 * (size_t)*ncl, cudaMemcpyHostToDevice,
                         ctx->st));
  } else {
    zeros.assign(*nl + 1, 0);
    CK(cudaMemcpyAsync(d.lm_cbeg, zeros.data(), 4 * (*nl + 1), cudaMemcpyHostToDevice, ctx->st));
  }
  CK(cudaStreamSynchronize(ctx->st));
  return SLOAM_OK;
}

int upload_ground(sloam_ctx* ctx, const float* g, int n) {
  if (n > ctx->d.cap_ground) return fail(ctx, SLOAM_ERR_CAPACITY, "ground points exceed capacity");
  if (n > 0)
    CK(cudaMemcpyAsync(ctx->d.ground, g, 16 * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
  return SLOAM_OK;
}

// planes + cylinders (+ features, inliers) into a sloam_models_out
int download_models(sloam_ctx* ctx, sloam_models_out* out) {
  Dev& d = ctx->d;
  const Counters& c = *ctx->h_cnt;
  out->n_planes = c.n_planes;
  out->n_cylinders = c.n_cyl;
  std::vector<PlaneD> pl(std::max(1, c.n_planes));
  std::vector<CylD> cy(std::max(1, c.n_cyl));
  if (c.n_planes)
    CK(cudaMemcpyAsync(pl.data(), d.planes, sizeof(PlaneD) * c.n_planes, cudaMemcpyDeviceToHost,
                       ctx->st));
  if (c.n_cyl)
    CK(cudaMemcpyAsync(cy.data(), d.cyls, sizeof(CylD) * c.n_cyl, cudaMemcpyDeviceToHost, ctx->st));
  std::vector<float4> feat((size_t)std::max(1, c.n_cyl) * std::max(1, d.F));
  if (c.n_cyl && out->cyl_features && d.F)
    CK(cudaMemcpyAsync(feat.data(), d.cyl_feat, sizeof(float4) * (size_t)c.n_cyl * d.F,
                       cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  const int np = std::min(c.n_planes, out->cap_planes);
  for (int k = 0; k < np && out->planes; ++k) {
    sloam_plane& o = out->planes[k];
    for (int j = 0; j < 4; ++j) o.plane[j] = pl[k].plane[j];
    for (int j = 0; j < 3; ++j) o.centroid[j] = pl[k].centroid[j];
    o.bin = pl[k].bin;
    o.valid = 1;
  }
  const int nc = std::min(c.n_cyl, out->cap_cylinders);
  for (int k = 0; k < nc && out->cylinders; ++k) {
    sloam_cylinder& o = out->cylinders[k];
    for (int j = 0; j < 3; ++j) {
      o.root[j] = cy[k].root[j];
      o.ray[j] = cy[k].ray[j];
    }
    o.radius = cy[k].radius;
    o.id = cy[k].id;
    o.valid = 1;
    if (out->cyl_inliers) out->cyl_inliers[k] = cy[k].inliers;
  }
  if (out->cyl_features && nc)
    std::memcpy(out->cyl_features, feat.data(), sizeof(float4) * (size_t)nc * d.F);
  if (c.n_planes > out->cap_planes || c.n_cyl > out->cap_cylinders)
    return fail(ctx, SLOAM_ERR_CAPACITY, "output capacity too small for the models");
  return SLOAM_OK;
}

void to_se3(const double* p, sloam_se3* s) {
  for (int j = 0; j < 4; ++j) s->q[j] = p[j];
  for (int j = 0; j < 3; ++j) s->t[j] = p[4 + j];
}

int download_run(sloam_ctx* ctx, sloam_run_out* out, bool first) {
  const Counters& c = *ctx->h_cnt;
  out->first_scan = first ? 1 : 0;
  out->success = c.success;
  out->n_tree_matches = c.n_tm;
  out->n_plane_matches = c.n_pm;
  out->tree_check = c.tree_check;
  out->ground_check = c.ground_check;
  to_se3(ctx->h_pose + 7, &out->T_Map_Curr);
  to_se3(ctx->h_pose + 14, &out->T_Delta);
  int st = download_models(ctx, &out->models);
  if (st) return st;
  const int nc = std::min(c.n_cyl, out->models.cap_cylinders);
  if (nc && out->matches)
    CK(cudaMemcpy(out->matches, ctx->d.match_out, 4 * (size_t)nc, cudaMemcpyDeviceToHost));
  return SLOAM_OK;
}

}  // namespace

// ================================================================== ABI
extern "C" sloam_ctx* sloam_create(const sloam_params* params, int device, int* status) {
  int dummy;
  if (!status) status = &dummy;
  if (!params || check_params(*params)) {
    *status = SLOAM_ERR_ARG;
    return nullptr;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    *status = SLOAM_ERR_NO_DEVICE;
    return nullptr;
  }
  sloam_ctx* ctx = new sloam_ctx;
  ctx->device = device;
  auto bail = [&](int code) {
    *status = code;
    sloam_destroy(ctx);
    return (sloam_ctx*)nullptr;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(SLOAM_ERR_NO_DEVICE);
  if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->fe_st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->fe_st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->fe_cp, cudaStreamNonBlocking) != cudaSuccess)
    return bail(SLOAM_ERR_CUDA);
  if (cudaMallocHost((void**)&ctx->h_cnt, sizeof(Counters)) != cudaSuccess ||
      cudaMallocHost((void**)&ctx->h_pose, sizeof(double) * 32) != cudaSuccess ||
      cudaMallocHost((void**)&ctx->h_in, sizeof(InPtrs) * 64) != cudaSuccess ||
      cudaMallocHost((void**)&ctx->h_poses, sizeof(double) * 8 * 64) != cudaSuccess)
    return bail(SLOAM_ERR_CUDA);
  ctx->h_batch_cap = 64;
  init_kernel_attributes();
  const int st = setup(ctx, *params);
  if (st != SLOAM_OK) return bail(st);
  *status = SLOAM_OK;
  return ctx;
}

extern "C" void sloam_destroy(sloam_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  destroy_graphs(ctx->gx);
  for (auto& s : ctx->extra) {
    if (s.st) cudaStreamSynchronize(s.st);
    destroy_graphs(s.gx);
    if (s.arena) cudaFree(s.arena);
    if (s.ev) cudaEventDestroy(s.ev);
    if (s.st) cudaStreamDestroy(s.st);
    destroy_fork(s.fk);
  }
  destroy_fork(ctx->fk);
  if (ctx->ev_main) cudaEventDestroy(ctx->ev_main);
  if (ctx->prop_tc) cudaFree(ctx->prop_tc);
  free_front(ctx);
  for (auto e : ctx->ev_fe) cudaEventDestroy(e);
  for (auto e : ctx->ev_cp) cudaEventDestroy(e);
  if (ctx->fe_st) cudaStreamDestroy(ctx->fe_st);
  if (ctx->fe_st2) cudaStreamDestroy(ctx->fe_st2);
  if (ctx->fe_cp) cudaStreamDestroy(ctx->fe_cp);
  if (ctx->d_out_i) cudaFree(ctx->d_out_i);
  if (ctx->d_out_pose) cudaFree(ctx->d_out_pose);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->h_cnt) cudaFreeHost(ctx->h_cnt);
  if (ctx->h_pose) cudaFreeHost(ctx->h_pose);
  if (ctx->h_in) cudaFreeHost(ctx->h_in);
  if (ctx->h_poses) cudaFreeHost(ctx->h_poses);
  if (ctx->d_in_all) cudaFree(ctx->d_in_all);
  if (ctx->d_poses_all) cudaFree(ctx->d_poses_all);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
}

extern "C" int sloam_last_error(const sloam_ctx* ctx, char* buf, size_t n) {
  if (!ctx || !buf || n == 0) return SLOAM_ERR_ARG;
  std::snprintf(buf, n, "%s", ctx->err.c_str());
  return SLOAM_OK;
}

extern "C" int sloam_reset(sloam_ctx* ctx) {
  if (!ctx) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  ctx->first_scan = true;
  CK(cudaMemsetAsync(ctx->d.cnt, 0, sizeof(Counters), ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return SLOAM_OK;
}

extern "C" int sloam_set_params(sloam_ctx* ctx, const sloam_params* params) {
  if (!ctx || !params || check_params(*params)) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->st));
  return setup(ctx, *params);
}

extern "C" int sloam_set_cc_iter_limit(sloam_ctx* ctx, int32_t limit) {
  if (!ctx) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->st));
  for (auto& s : ctx->extra) CK(cudaStreamSynchronize(s.st));
  ctx->cc_iter_limit = limit < 0 ? -1 : limit;
  ctx->kp.cc_iter_limit = limit < 0 ? kCCIterLimitDefault : limit;
  // the captured keyframe graphs hold the old value: capture again
  destroy_graphs(ctx->gx);
  for (auto& s : ctx->extra) destroy_graphs(s.gx);
  return SLOAM_OK;
}

extern "C" int64_t sloam_last_launch_count(const sloam_ctx* ctx) {
  return ctx ? ctx->last_launches : 0;
}
extern "C" void* sloam_stream(sloam_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }

// ----------------------------------------------------------- a1/a2
extern "C" int sloam_project_mask(sloam_ctx* ctx, const float* xyzi, int32_t n,
                                  const uint8_t* point_labels, const uint8_t* mask_image,
                                  sloam_scan_out* out) {
  if (!ctx || !xyzi || !out || (!point_labels && !mask_image)) return SLOAM_ERR_ARG;
  Dev& d = ctx->d;
  if (n != d.N) return fail(ctx, SLOAM_ERR_ARG, "n must equal img_h * img_w");
  cudaSetDevice(ctx->device);
  CK(cudaMemcpyAsync(d.buf_xyzi, xyzi, 16 * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
  if (point_labels)
    CK(cudaMemcpyAsync(d.buf_plabel, point_labels, n, cudaMemcpyHostToDevice, ctx->st));
  else
    CK(cudaMemcpyAsync(d.buf_mask_in, mask_image, n, cudaMemcpyHostToDevice, ctx->st));
  int st = set_inputs(ctx, d.buf_xyzi, d.buf_plabel, d.buf_mask_in, d.buf_map, 0);
  if (st) return st;
  int nl = launch_begin(d, -1, 0, 0, 0, 0, ctx->st);
  nl += launch_project(d, ctx->kp, point_labels != nullptr, ctx->st);
  ctx->last_launches = nl;
  st = sync_counters(ctx);
  if (st) return st;
  const int ng = ctx->h_cnt->n_ground;
  out->n_ground = ng;
  if (out->px || out->py) {
    std::vector<int32_t> pix(n);
    CK(cudaMemcpy(pix.data(), d.pix, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
      if (out->px) out->px[i] = pix[i] % d.W;
      if (out->py) out->py[i] = pix[i] / d.W;
    }
  }
  if (out->range_image)
    CK(cudaMemcpy(out->range_image, d.range_img, 4 * (size_t)n, cudaMemcpyDeviceToHost));
  if (out->mask_out) CK(cudaMemcpy(out->mask_out, d.mask, n, cudaMemcpyDeviceToHost));
  if (out->ground_idx && ng)
    CK(cudaMemcpy(out->ground_idx, d.ground_idx, 4 * (size_t)ng, cudaMemcpyDeviceToHost));
  if (out->tree_cloud)
    CK(cudaMemcpy(out->tree_cloud, d.tree, 16 * (size_t)n, cudaMemcpyDeviceToHost));
  return SLOAM_OK;
}

// --------------------------------------------------------------- a3-a5
extern "C" int sloam_trellis(sloam_ctx* ctx, const float* tree_cloud, int32_t H, int32_t W,
                             uint32_t* cc_labels, int32_t* n_components, sloam_landmarks* out) {
  if (!ctx || !tree_cloud || !out) return SLOAM_ERR_ARG;
  Dev& d = ctx->d;
  if (H != d.H || W != d.W) return fail(ctx, SLOAM_ERR_ARG, "H, W must match the context");
  cudaSetDevice(ctx->device);
  CK(cudaMemcpyAsync(d.tree, tree_cloud, 16 * (size_t)d.N, cudaMemcpyHostToDevice, ctx->st));
  int st = set_inputs(ctx, nullptr, nullptr, nullptr, nullptr, 0);
  if (st) return st;
  int nl = launch_begin(d, 0, -1, -1, -1, -1, ctx->st);
  nl += launch_trellis(d, ctx->kp, ctx->st);
  ctx->last_launches = nl;
  if ((st = sync_counters(ctx))) return st;
  const Counters& c = *ctx->h_cnt;
  if (n_components) *n_components = c.n_comp;
  if (cc_labels) CK(cudaMemcpy(cc_labels, d.label, 4 * (size_t)d.N, cudaMemcpyDeviceToHost));
  out->n_landmarks = c.n_lm;
  out->n_vertices = c.n_v;
  out->n_points = c.n_p;
  out->n_cluster = c.n_cluster;
  if (c.n_lm > out->cap_landmarks || c.n_v > out->cap_vertices || c.n_p > out->cap_points)
    return fail(ctx, SLOAM_ERR_CAPACITY, "landmark output capacity too small");
  if (c.n_lm) {
    CK(cudaMemcpy(out->tree_id, d.lm_tree, 4 * (size_t)c.n_lm, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out->vertex_begin, d.lm_vbeg, 4 * (size_t)(c.n_lm + 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out->vertex_xyz, d.lm_vxyz, 12 * (size_t)c.n_v, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out->vertex_radius, d.lm_vrad, 8 * (size_t)c.n_v, cudaMemcpyDeviceToHost));
    if (out->vertex_row)
      CK(cudaMemcpy(out->vertex_row, d.lm_vrow, 4 * (size_t)c.n_v, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out->point_begin, d.lm_pbeg, 4 * (size_t)(c.n_v + 1), cudaMemcpyDeviceToHost));
    if (c.n_p)
      CK(cudaMemcpy(out->point_xyzi, d.lm_pts, 16 * (size_t)c.n_p, cudaMemcpyDeviceToHost));
    if (out->cluster_begin) {
      if (c.n_cluster > out->cap_cluster)
        return fail(ctx, SLOAM_ERR_CAPACITY, "cluster output capacity too small");
      CK(cudaMemcpy(out->cluster_begin, d.lm_cbeg, 4 * (size_t)(c.n_lm + 1),
                    cudaMemcpyDeviceToHost));
      if (out->cluster_xyzi && c.n_cluster)
        CK(cudaMemcpy(out->cluster_xyzi, d.lm_cpts, 16 * (size_t)c.n_cluster,
                      cudaMemcpyDeviceToHost));
    }
  } else {
    out->vertex_begin[0] = 0;
    if (out->cluster_begin) out->cluster_begin[0] = 0;
  }
  return SLOAM_OK;
}

// --------------------------------------------------------------- a6-a8
extern "C" int sloam_compute_models(sloam_ctx* ctx, const sloam_se3* pose,
                                    const float* ground_xyzi, int32_t n_ground,
                                    const sloam_landmarks* lm, sloam_models_out* out) {
  if (!ctx || !pose || !out || (n_ground > 0 && !ground_xyzi) || n_ground < 0)
    return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  int nl, nv, np, ncl;
  int st = upload_landmarks(ctx, lm, &nl, &nv, &np, &ncl);
  if (st) return st;
  if ((st = upload_ground(ctx, ground_xyzi, n_ground))) return st;
  if ((st = upload_pose(ctx, pose))) return st;
  if ((st = set_inputs(ctx, nullptr, nullptr, nullptr, nullptr, 0))) return st;
  int k = launch_begin(d, n_ground, nl, nv, np, ncl, ctx->st);
  k += launch_models(d, ctx->kp, false, ctx->st);
  ctx->last_launches = k;
  if ((st = sync_counters(ctx))) return st;
  return download_models(ctx, out);
}

extern "C" int sloam_fit_plane(sloam_ctx* ctx, const float* xyzi, int32_t n, sloam_plane* out,
                               float* features) {
  if (!ctx || !out || n < 0 || (n > 0 && !xyzi)) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  Dev& d = ctx->d;
  if (n > d.cap_ground) return fail(ctx, SLOAM_ERR_CAPACITY, "more points than max_ground");
  int st = upload_ground(ctx, xyzi, n);
  if (st || (st = set_inputs(ctx, nullptr, nullptr, nullptr, nullptr, 0))) return st;
  int k = launch_begin(d, n, -1, -1, -1, -1, ctx->st);
  k += launch_plane_points(d, ctx->kp, n, ctx->st);
  ctx->last_launches = k;
  if ((st = sync_counters(ctx))) return st;
  PlaneD pl;
  CK(cudaMemcpy(&pl, d.plane_all, sizeof(PlaneD), cudaMemcpyDeviceToHost));
  for (int j = 0; j < 4; ++j) out->plane[j] = pl.plane[j];
  for (int j = 0; j < 3; ++j) out->centroid[j] = pl.centroid[j];
  out->bin = pl.bin;
  out->valid = pl.valid;
  if (features && pl.valid && d.G > 0)
    CK(cudaMemcpy(features, d.plane_feat_all, sizeof(float4) * d.G, cudaMemcpyDeviceToHost));
  return SLOAM_OK;
}

extern "C" int sloam_fit_cylinders(sloam_ctx* ctx, const sloam_landmarks* lm,
                                   const sloam_plane* planes, int32_t n_planes,
                                   sloam_models_out* out) {
  if (!ctx || !lm || !out || n_planes < 0 || (n_planes > 0 && !planes)) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  if (n_planes > d.n_bins) return fail(ctx, SLOAM_ERR_CAPACITY, "more planes than ground bins");
  int nl, nv, np, ncl;
  int st = upload_landmarks(ctx, lm, &nl, &nv, &np, &ncl);
  if (st || (st = set_inputs(ctx, nullptr, nullptr, nullptr, nullptr, 0))) return st;
  std::vector<PlaneD> pl(std::max(1, (int)n_planes));
  for (int k = 0; k < n_planes; ++k) {
    for (int j = 0; j < 4; ++j) pl[k].plane[j] = planes[k].plane[j];
    for (int j = 0; j < 3; ++j) pl[k].centroid[j] = planes[k].centroid[j];
    pl[k].bin = planes[k].bin;
    pl[k].valid = 1;
  }
  int k = launch_begin(d, 0, nl, nv, np, ncl, ctx->st);
  if (n_planes)
    CK(cudaMemcpyAsync(d.planes, pl.data(), sizeof(PlaneD) * n_planes, cudaMemcpyHostToDevice,
                       ctx->st));
  CK(cudaMemcpyAsync(&d.cnt->n_planes, &n_planes, sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->st));
  k += launch_cylinders(d, ctx->kp, false, ctx->st);
  ctx->last_launches = k;
  if ((st = sync_counters(ctx))) return st;
  return download_models(ctx, out);
}

// ---------------------------------------------------------------- a9-a11
extern "C" int sloam_run(sloam_ctx* ctx, const sloam_se3* pose, const float* ground_xyzi,
                         int32_t n_ground, const sloam_landmarks* lm, const sloam_cylinder* map,
                         int32_t n_map, sloam_run_out* out) {
  if (!ctx || !pose || !out || n_ground < 0 || n_map < 0 || (n_map > 0 && !map))
    return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  const bool first = ctx->first_scan;
  if (!first && n_map == 0) {
    out->success = 0;
    return fail(ctx, SLOAM_ERR_EMPTY_MAP, "not the first scan but the map is empty");
  }
  if (n_map > d.cap_map) return fail(ctx, SLOAM_ERR_CAPACITY, "map exceeds max_map");
  int nl, nv, np, ncl;
  int st = upload_landmarks(ctx, lm, &nl, &nv, &np, &ncl);
  if (st) return st;
  if ((st = upload_ground(ctx, ground_xyzi, n_ground))) return st;
  if (n_map)
    CK(cudaMemcpyAsync(d.buf_map, map, sizeof(sloam_cylinder) * n_map, cudaMemcpyHostToDevice,
                       ctx->st));
  if ((st = set_inputs(ctx, d.buf_xyzi, d.buf_plabel, d.buf_mask_in, d.buf_map, n_map))) return st;
  if ((st = upload_pose(ctx, pose))) return st;
  int k = launch_begin(d, n_ground, nl, nv, np, ncl, ctx->st);
  k += launch_models(d, ctx->kp, false, ctx->st);
  k += launch_run(d, ctx->kp, first, true, ctx->st);
  ctx->last_launches = k;
  if ((st = sync_counters(ctx))) return st;
  ctx->first_scan = false;
  const int status = first ? SLOAM_OK : ctx->h_cnt->status;
  if (status == SLOAM_ERR_NO_MODELS) {
    out->success = 0;
    return fail(ctx, SLOAM_ERR_NO_MODELS, "no ground or landmark models found");
  }
  if ((st = download_run(ctx, out, first))) return st;
  return status;
}

// ----------------------------------------------------------- keyframe
namespace {
// The ground planes need only the ground list, the submap prep only the map
// input, the Trellis and the cylinder fits only the tree cloud: the planes
// and the submap prep run on the slot's aux stream beside them (a fork and
// a join in the captured graph), and the plane gates, the cylinder list and
// the pose follow once both are done.  -1: a fork call failed.
int enqueue_keyframe(sloam_ctx* ctx, const Dev& d, cudaStream_t st, const Fork& fk, bool first,
                     bool point_labels, bool update, bool pre) {
  int k = launch_begin(d, -1, -1, -1, -1, -1, st);
  if (!pre) k += launch_project(d, ctx->kp, point_labels, st);
  if (cudaEventRecord(fk.fork, st) != cudaSuccess ||
      cudaStreamWaitEvent(fk.aux, fk.fork, 0) != cudaSuccess)
    return -1;
  k += launch_planes(d, ctx->kp, fk.aux);
  if (!first) k += launch_map_prep(d, fk.aux);  // the submap needs the map input only
  if (cudaEventRecord(fk.join, fk.aux) != cudaSuccess) return -1;
  k += launch_trellis(d, ctx->kp, st);
  k += launch_cylinder_fits(d, ctx->kp, true, st);
  if (cudaStreamWaitEvent(st, fk.join, 0) != cudaSuccess) return -1;
  k += launch_cylinder_close(d, ctx->kp, st);
  k += launch_run(d, ctx->kp, first, update, st, true);
  return k;
}

// The whole keyframe (a1-a11, or a3-a11 when a batch launch did the
// projection) of one slot as one CUDA graph, captured on first use; returns
// the number of kernels it launches in *nk.
int run_graph(sloam_ctx* ctx, const Dev& d, cudaStream_t st, const Fork& fk, GraphSet& gs,
              bool first, bool point_labels, bool update, bool pre, int* nk) {
  const int a = first ? 1 : 0, b = point_labels ? 1 : 0, u = update ? 1 : 0, q = pre ? 1 : 0;
  cudaGraphExec_t& gx = gs.g[a][b][u][q];
  if (!gx) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int k = enqueue_keyframe(ctx, d, st, fk, first, point_labels, update, pre);
    CK(cudaStreamEndCapture(st, &g));
    if (k < 0) {
      cudaGraphDestroy(g);
      return fail(ctx, SLOAM_ERR_CUDA, "keyframe graph: fork or join of the aux stream");
    }
    cudaError_t e = cudaGraphInstantiate(&gx, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ctx, SLOAM_ERR_CUDA, "cudaGraphInstantiate", e);
    gs.launches[a][b][u][q] = k;
  }
  CK(cudaGraphLaunch(gx, st));
  *nk = gs.launches[a][b][u][q];
  return SLOAM_OK;
}

int run_keyframe_graph(sloam_ctx* ctx, bool first, bool point_labels, bool update) {
  int nk = 0;
  const int s =
      run_graph(ctx, ctx->d, ctx->st, ctx->fk, ctx->gx, first, point_labels, update, false, &nk);
  ctx->last_launches = nk;
  return s;
}
}  // namespace

extern "C" int sloam_keyframe(sloam_ctx* ctx, const float* xyzi, int32_t n,
                              const uint8_t* point_labels, const uint8_t* mask_image,
                              const sloam_se3* pose, const sloam_cylinder* map, int32_t n_map,
                              sloam_run_out* out) {
  if (!ctx || !xyzi || !pose || !out || (!point_labels && !mask_image) || n_map < 0 ||
      (n_map > 0 && !map))
    return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  if (n != d.N) return fail(ctx, SLOAM_ERR_ARG, "n must equal img_h * img_w");
  const bool first = ctx->first_scan;
  if (!first && n_map == 0) {
    out->success = 0;
    return fail(ctx, SLOAM_ERR_EMPTY_MAP, "not the first scan but the map is empty");
  }
  if (n_map > d.cap_map) return fail(ctx, SLOAM_ERR_CAPACITY, "map exceeds max_map");
  CK(cudaMemcpyAsync(d.buf_xyzi, xyzi, 16 * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
  if (point_labels)
    CK(cudaMemcpyAsync(d.buf_plabel, point_labels, n, cudaMemcpyHostToDevice, ctx->st));
  else
    CK(cudaMemcpyAsync(d.buf_mask_in, mask_image, n, cudaMemcpyHostToDevice, ctx->st));
  if (n_map)
    CK(cudaMemcpyAsync(d.buf_map, map, sizeof(sloam_cylinder) * n_map, cudaMemcpyHostToDevice,
                       ctx->st));
  int st = set_inputs(ctx, d.buf_xyzi, d.buf_plabel, d.buf_mask_in, d.buf_map, n_map);
  if (st) return st;
  if ((st = upload_pose(ctx, pose))) return st;
  if ((st = run_keyframe_graph(ctx, first, point_labels != nullptr, true))) return st;
  if ((st = sync_counters(ctx))) return st;
  ctx->first_scan = false;
  const int status = first ? SLOAM_OK : ctx->h_cnt->status;
  if (status == SLOAM_ERR_NO_MODELS) {
    out->success = 0;
    return fail(ctx, SLOAM_ERR_NO_MODELS, "no ground or landmark models found");
  }
  if ((st = download_run(ctx, out, first))) return st;
  return status;
}

extern "C" int sloam_keyframe_mapped(sloam_ctx* ctx, sloam_mapmgr* mm, const float* xyzi,
                                     int32_t n, const uint8_t* point_labels,
                                     const uint8_t* mask_image, const sloam_se3* pose,
                                     sloam_run_out* out) {
  if (!ctx || !mm || !xyzi || !pose || !out || (!point_labels && !mask_image))
    return SLOAM_ERR_ARG;
  if (sg::mapmgr_device(mm) != ctx->device)
    return fail(ctx, SLOAM_ERR_ARG, "the map manager is on another device");
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  const sg::MapMgrDev& m = sg::mapmgr_dev(mm);
  if (n != d.N) return fail(ctx, SLOAM_ERR_ARG, "n must equal img_h * img_w");
  if (m.k > d.cap_map) return fail(ctx, SLOAM_ERR_CAPACITY, "submap size k exceeds max_map");
  const bool first = ctx->first_scan;
  CK(cudaMemcpyAsync(d.buf_xyzi, xyzi, 16 * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
  if (point_labels)
    CK(cudaMemcpyAsync(d.buf_plabel, point_labels, n, cudaMemcpyHostToDevice, ctx->st));
  else
    CK(cudaMemcpyAsync(d.buf_mask_in, mask_image, n, cudaMemcpyHostToDevice, ctx->st));
  int st = set_inputs(ctx, d.buf_xyzi, d.buf_plabel, d.buf_mask_in, m.sub, 0);
  if (st) return st;
  if ((st = upload_pose(ctx, pose))) return st;
  // getSubmap on the device; map and n_map of the input block follow it
  sg::launch_mm_submap(m, pose->t[0], pose->t[1], d.in, ctx->st);
  int32_t n_sub = 0;
  CK(cudaMemcpyAsync(&ctx->h_cnt->pad[0], m.state + 1, 4, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  n_sub = ctx->h_cnt->pad[0];
  if (!first && n_sub == 0) {
    out->success = 0;
    return fail(ctx, SLOAM_ERR_EMPTY_MAP, "not the first scan but the submap is empty");
  }
  if ((st = run_keyframe_graph(ctx, first, point_labels != nullptr, true))) return st;
  int nk = ctx->last_launches;
  nk += sg::launch_mm_update(m, d, first ? 1 : 0, ctx->st);
  ctx->last_launches = nk + 1;
  if ((st = sync_counters(ctx))) return st;
  ctx->first_scan = false;
  const int status = first ? SLOAM_OK : ctx->h_cnt->status;
  if (status == SLOAM_ERR_NO_MODELS) {
    out->success = 0;
    return fail(ctx, SLOAM_ERR_NO_MODELS, "no ground or landmark models found");
  }
  if ((st = download_run(ctx, out, first))) return st;
  return status;
}

namespace sg {
// keyframe k's input block and pose estimate, from the batch's device copies
// into its slot
static_assert(sizeof(InPtrs) % 8 == 0, "InPtrs copied as 8-byte words");
__global__ void k_batch_in(const InPtrs* __restrict__ all_in, const double* __restrict__ all_pose,
                           int k, InPtrs* in, double* pose_io) {
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(all_in + k);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(in);
  for (int i = threadIdx.x; i < (int)(sizeof(InPtrs) / 8); i += blockDim.x) dst[i] = src[i];
  if (threadIdx.x < 7) pose_io[threadIdx.x] = all_pose[8 * k + threadIdx.x];
}
// per-keyframe outputs of a device batch
__global__ void k_batch_out(Counters* c, const double* pose_io, double* pose_out,
                            int32_t* success_out, int32_t* ncyl_out, int k) {
  if (threadIdx.x < 7) pose_out[7 * k + threadIdx.x] = pose_io[7 + threadIdx.x];
  if (threadIdx.x == 0) {
    // a keyframe where a bounded wait gave up is not a success
    const bool gave_up = c->cc_iter_exceeded || c->prop_err || c->queue_err;
    success_out[k] = (c->status == SLOAM_OK && !gave_up) ? c->success : 0;
    ncyl_out[k] = c->n_cyl;
  }
}
}  // namespace sg

namespace {
// A keyframe slot of a batch: slot 0 is the context's own state.
struct SlotView {
  Dev* d;
  cudaStream_t st;
  GraphSet* gx;
  cudaEvent_t ev;
  const Fork* fk;
};
SlotView slot(sloam_ctx* ctx, int s) {
  if (s == 0) return {&ctx->d, ctx->st, &ctx->gx, nullptr, &ctx->fk};
  auto& x = ctx->extra[s - 1];
  return {&x.d, x.st, &x.gx, x.ev, &x.fk};
}

int grow_batch(sloam_ctx* ctx, int nkf) {
  if (nkf > ctx->h_batch_cap) {
    cudaFreeHost(ctx->h_in);
    cudaFreeHost(ctx->h_poses);
    ctx->h_in = nullptr;
    ctx->h_poses = nullptr;
    CK(cudaMallocHost((void**)&ctx->h_in, sizeof(InPtrs) * nkf));
    CK(cudaMallocHost((void**)&ctx->h_poses, sizeof(double) * 8 * nkf));
    ctx->h_batch_cap = nkf;
  }
  if (ctx->d_batch_cap < ctx->h_batch_cap) {
    if (ctx->d_in_all) cudaFree(ctx->d_in_all);
    if (ctx->d_poses_all) cudaFree(ctx->d_poses_all);
    ctx->d_in_all = nullptr;
    ctx->d_poses_all = nullptr;
    CK(cudaMalloc((void**)&ctx->d_in_all, sizeof(InPtrs) * ctx->h_batch_cap));
    CK(cudaMalloc((void**)&ctx->d_poses_all, sizeof(double) * 8 * ctx->h_batch_cap));
    ctx->d_batch_cap = ctx->h_batch_cap;
  }
  return SLOAM_OK;
}

// One keyframe's projection outputs inside the batch buffers (the scan
// upload space last, when present).  The point pixels and pixel keys are
// scratch of the chunk in flight (fb_pix, fb_pkey), small enough to stay in
// L2 between the chunk's kernels.
struct FrontSlice {
  FrontRef f{};
  float4* up_xyzi = nullptr;
  uint8_t* up_plabel = nullptr;
};
FrontSlice front_slice(const Dev& d, char* base, bool upload, size_t* bytes) {
  Carver c{base, 0, base == nullptr};
  const int N = d.N;
  FrontSlice s;
  s.f.range_img = c.take<float>(N);
  s.f.mask = c.take<uint8_t>(N);
  // the tree cloud and the ground list stay views of the scan: a tree flag
  // per point and the ground point indices (no 16 B copies per point)
  s.f.tree = nullptr;
  s.f.tflag = c.take<uint8_t>(N);
  s.f.gbits = c.take<uint32_t>(front_gbits_words(N));
  s.f.blk = c.take<int32_t>(front_blocks(N));  // ground count per 1024-point chunk
  s.f.ground_idx = c.take<int32_t>(N);
  s.f.ground = nullptr;
  if (upload) {
    s.up_xyzi = c.take<float4>(N);
    s.up_plabel = c.take<uint8_t>(N);
  }
  if (bytes) *bytes = (c.off + 255) & ~(size_t)255;
  return s;
}

void free_front(sloam_ctx* ctx) {
  if (ctx->fe_cp) cudaStreamSynchronize(ctx->fe_cp);
  if (ctx->fe_st) cudaStreamSynchronize(ctx->fe_st);
  if (ctx->fe_st2) cudaStreamSynchronize(ctx->fe_st2);
  if (ctx->fb) cudaFree(ctx->fb);
  if (ctx->fb_pix) cudaFree(ctx->fb_pix);
  if (ctx->fb_pkey) cudaFree(ctx->fb_pkey);
  if (ctx->d_refs) cudaFree(ctx->d_refs);
  if (ctx->fb_fe) cudaFree(ctx->fb_fe);
  if (ctx->h_refs) cudaFreeHost(ctx->h_refs);
  ctx->fb = nullptr;
  ctx->fb_pix = nullptr;
  ctx->fb_pkey = nullptr;
  ctx->d_refs = nullptr;
  ctx->fb_fe = nullptr;
  ctx->h_refs = nullptr;
  ctx->fb_cap = 0;
  ctx->fb_upload = false;
}

// Batch projection buffers for nkf keyframes (kept and reused; the pixel
// keys start all-ones and every chunk re-arms them).
int grow_front(sloam_ctx* ctx, int nkf, bool upload) {
  if (nkf <= ctx->fb_cap && (!upload || ctx->fb_upload)) return SLOAM_OK;
  const int cap = std::max(nkf, ctx->fb_cap);
  upload = upload || ctx->fb_upload;
  free_front(ctx);
  size_t stride = 0;
  front_slice(ctx->d, nullptr, upload, &stride);
  CK(cudaMalloc(&ctx->fb, stride * cap));
  const size_t sn = (size_t)2 * kFrontChunkMax * ctx->d.N;  // two sets
  CK(cudaMalloc((void**)&ctx->fb_pix, sizeof(int32_t) * sn));
  CK(cudaMalloc((void**)&ctx->fb_pkey, sizeof(unsigned long long) * sn));
  CK(cudaMemsetAsync(ctx->fb_pkey, 0xFF, sizeof(unsigned long long) * sn, ctx->fe_st));
  CK(cudaMalloc((void**)&ctx->d_refs, sizeof(FrontRef) * cap));
  CK(cudaMalloc((void**)&ctx->fb_fe, sizeof(int32_t) * 4 * cap));
  CK(cudaMallocHost((void**)&ctx->h_refs, sizeof(FrontRef) * cap));
  ctx->fb_stride = stride;
  ctx->fb_cap = cap;
  ctx->fb_upload = upload;
  CK(cudaStreamSynchronize(ctx->fe_st));
  return SLOAM_OK;
}

// Fork: the projection stream and every extra slot wait for the context
// stream; the extra slots take a copy of the previous-scan planes (the batch
// does not advance the state).
int batch_fork(sloam_ctx* ctx) {
  CK(cudaEventRecord(ctx->ev_main, ctx->st));
  CK(cudaStreamWaitEvent(ctx->fe_st, ctx->ev_main, 0));
  for (auto& s : ctx->extra) {
    CK(cudaStreamWaitEvent(s.st, ctx->ev_main, 0));
    CK(cudaMemcpyAsync(s.d.prev_planes, ctx->d.prev_planes, sizeof(PlaneD) * ctx->d.n_bins,
                       cudaMemcpyDeviceToDevice, s.st));
    CK(cudaMemcpyAsync(&s.d.cnt->n_prev, &ctx->d.cnt->n_prev, sizeof(int32_t),
                       cudaMemcpyDeviceToDevice, s.st));
  }
  return SLOAM_OK;
}
// Join: the context stream waits for every slot and the projection stream.
int batch_join(sloam_ctx* ctx) {
  for (auto& s : ctx->extra) {
    CK(cudaEventRecord(s.ev, s.st));
    CK(cudaStreamWaitEvent(ctx->st, s.ev, 0));
  }
  if (ctx->fe_chunks > 0)
    CK(cudaStreamWaitEvent(ctx->st, ctx->ev_fe[3 * ctx->fe_chunks - 1], 0));
  return SLOAM_OK;
}

// Keyframe k of a batch on slot k % slots: inputs pointer block and pose
// estimate from pinned host memory, the slot's graph (projection already
// done, no state update), then its outputs into the batch arrays.
int batch_one(sloam_ctx* ctx, int k, double* pose_out, int32_t* success_out, int32_t* ncyl_out,
              int64_t* launches) {
  const int S = 1 + (int)ctx->extra.size();
  SlotView v = slot(ctx, k % S);
  k_batch_in<<<1, 32, 0, v.st>>>(ctx->d_in_all, ctx->d_poses_all, k, v.d->in, v.d->pose_io);
  int nk = 0;
  int st = run_graph(ctx, *v.d, v.st, *v.fk, *v.gx, false, true, false, true, &nk);
  if (st) return st;
  k_batch_out<<<1, 32, 0, v.st>>>(v.d->cnt, v.d->pose_io, pose_out, success_out, ncyl_out, k);
  *launches += nk + 2;
  return SLOAM_OK;
}

void fill_pose(sloam_ctx* ctx, int k, const sloam_se3& p) {
  for (int j = 0; j < 4; ++j) ctx->h_poses[8 * k + j] = p.q[j];
  for (int j = 0; j < 3; ++j) ctx->h_poses[8 * k + 4 + j] = p.t[j];
}

// Per-keyframe projection views and input blocks of a batch.  Scans come
// from the caller's device arrays (xyzi, labels) or, when those are null,
// from the upload space of the batch buffers.
void fill_batch(sloam_ctx* ctx, int nkf, const float* xyzi, const uint8_t* labels,
                const sloam_se3* poses, const sloam_cylinder* d_map, int n_map) {
  const int n = ctx->d.N;
  ctx->fe_chunk = xyzi ? kFrontChunkDevice : kFrontChunkHost;
  for (int k = 0; k < nkf; ++k) {
    FrontSlice s = front_slice(ctx->d, (char*)ctx->fb + ctx->fb_stride * k, ctx->fb_upload,
                               nullptr);
    FrontRef& f = ctx->h_refs[k];
    f = s.f;
    // chunk scratch: set (chunk & 1), slot k % chunk
    const size_t sc = (size_t)((k / ctx->fe_chunk) & 1) * kFrontChunkMax + k % ctx->fe_chunk;
    f.pix = ctx->fb_pix + sc * n;
    f.pkey = ctx->fb_pkey + sc * n;
    f.xyzi = xyzi ? reinterpret_cast<const float4*>(xyzi) + (size_t)k * n : s.up_xyzi;
    f.plabel = labels ? labels + (size_t)k * n : s.up_plabel;
    f.mask_in = nullptr;
    f.fe = ctx->fb_fe + 4 * k;
    InPtrs& h = ctx->h_in[k];
    h.xyzi = f.xyzi;
    h.plabel = f.plabel;
    h.mask_in = nullptr;
    h.map = d_map;
    h.tree = nullptr;
    h.ground = nullptr;
    h.fe = f.fe;
    h.tflag = f.tflag;
    h.gidx = f.ground_idx;
    h.n_map = n_map;
    h.destag = ctx->kp.do_destagger ? 1 : 0;
    fill_pose(ctx, k, poses[k]);
  }
}

// The batch: projection of each chunk of keyframes on the projection stream,
// then the keyframes on their slots.  Host input: each chunk's scans are
// uploaded before its projection, and a slot waits only for the chunk of its
// keyframe, so uploads, projection and the slots overlap.  Device input: the
// slots wait for the last chunk, so the projection runs alone on the GPU.
int batch_run(sloam_ctx* ctx, int nkf, const float* h_xyzi, const uint8_t* h_labels,
              double* pose_out, int32_t* success_out, int32_t* ncyl_out, int64_t* launches) {
  const int n = ctx->d.N;
  const int S = 1 + (int)ctx->extra.size();
  const int chunk = ctx->fe_chunk;
  const int nch = (nkf + chunk - 1) / chunk;
  while ((int)ctx->ev_fe.size() < 3 * nch) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    ctx->ev_fe.push_back(e);
  }
  while (h_xyzi && (int)ctx->ev_cp.size() < nch) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->ev_cp.push_back(e);
  }
  // the uploads start once the batch has forked from the context stream;
  // first the keyframes' input blocks and pose estimates (each slot waits
  // for its keyframe's chunk, whose projection comes after them on either
  // path)
  cudaStream_t up = h_xyzi ? ctx->fe_cp : ctx->fe_st;
  if (h_xyzi) CK(cudaStreamWaitEvent(ctx->fe_cp, ctx->ev_main, 0));
  CK(cudaMemcpyAsync(ctx->d_in_all, ctx->h_in, sizeof(InPtrs) * nkf, cudaMemcpyHostToDevice, up));
  CK(cudaMemcpyAsync(ctx->d_poses_all, ctx->h_poses, sizeof(double) * 8 * nkf,
                     cudaMemcpyHostToDevice, up));
  CK(cudaMemcpyAsync(ctx->d_refs, ctx->h_refs, sizeof(FrontRef) * nkf, cudaMemcpyHostToDevice,
                     ctx->fe_st));
  CK(cudaMemsetAsync(ctx->fb_fe, 0, sizeof(int32_t) * 4 * nkf, ctx->fe_st));
  ctx->fe_chunks = 0;
  for (int c = 0; c < nch; ++c) {
    const int kf0 = c * chunk, nc = std::min(chunk, nkf - kf0);
    if (h_xyzi) {
      for (int k = kf0; k < kf0 + nc; ++k) {
        FrontRef& f = ctx->h_refs[k];
        CK(cudaMemcpyAsync(const_cast<float4*>(f.xyzi), h_xyzi + (size_t)k * n * 4,
                           16 * (size_t)n, cudaMemcpyHostToDevice, ctx->fe_cp));
        CK(cudaMemcpyAsync(const_cast<uint8_t*>(f.plabel), h_labels + (size_t)k * n, (size_t)n,
                           cudaMemcpyHostToDevice, ctx->fe_cp));
      }
      CK(cudaEventRecord(ctx->ev_cp[c], ctx->fe_cp));
      CK(cudaStreamWaitEvent(ctx->fe_st, ctx->ev_cp[c], 0));
    }
    // the scratch set of chunk c - 2 is re-armed by that chunk's compaction
    if (c >= 2) CK(cudaStreamWaitEvent(ctx->fe_st, ctx->ev_fe[3 * (c - 2) + 2], 0));
    CK(cudaEventRecord(ctx->ev_fe[3 * c], ctx->fe_st));
    *launches += launch_project_batch_points(ctx->d, ctx->kp, ctx->d_refs, kf0, nc, true,
                                             ctx->fe_st);
    CK(cudaEventRecord(ctx->ev_fe[3 * c + 1], ctx->fe_st));
    CK(cudaStreamWaitEvent(ctx->fe_st2, ctx->ev_fe[3 * c + 1], 0));
    *launches += launch_project_batch_labels(ctx->d, ctx->d_refs, kf0, nc, true, ctx->fe_st2);
    CK(cudaEventRecord(ctx->ev_fe[3 * c + 2], ctx->fe_st2));
    ctx->fe_chunks = c + 1;
    if (!h_xyzi) continue;
    for (int k = kf0; k < kf0 + nc; ++k) {
      CK(cudaStreamWaitEvent(slot(ctx, k % S).st, ctx->ev_fe[3 * c + 2], 0));
      int st = batch_one(ctx, k, pose_out, success_out, ncyl_out, launches);
      if (st) return st;
    }
  }
  ctx->fe_nkf = nkf;
  if (h_xyzi || nch == 0) return SLOAM_OK;
  for (int s = 0; s < S && s < nkf; ++s)
    CK(cudaStreamWaitEvent(slot(ctx, s).st, ctx->ev_fe[3 * nch - 1], 0));
  for (int k = 0; k < nkf; ++k) {
    int st = batch_one(ctx, k, pose_out, success_out, ncyl_out, launches);
    if (st) return st;
  }
  return SLOAM_OK;
}
}  // namespace

extern "C" int sloam_keyframes_device(sloam_ctx* ctx, const float* d_xyzi, int32_t n,
                                      int32_t nkf, const uint8_t* d_point_labels,
                                      const sloam_se3* poses, const sloam_cylinder* d_map,
                                      int32_t n_map, double* d_pose_out, int32_t* d_success_out,
                                      int32_t* d_ncyl_out) {
  if (!ctx || !d_xyzi || !d_point_labels || !poses || nkf < 0 || !d_pose_out ||
      !d_success_out || !d_ncyl_out || n_map <= 0 || !d_map)
    return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  if (n != d.N) return fail(ctx, SLOAM_ERR_ARG, "n must equal img_h * img_w");
  if (ctx->first_scan) return fail(ctx, SLOAM_ERR_ARG, "the context has not seen a first scan");
  if (n_map > d.cap_map) return fail(ctx, SLOAM_ERR_CAPACITY, "map exceeds max_map");
  CK(cudaStreamSynchronize(ctx->st));  // the previous batch released the pinned blocks
  int st = grow_batch(ctx, nkf);
  if (st || (st = grow_front(ctx, nkf, false))) return st;
  fill_batch(ctx, nkf, d_xyzi, d_point_labels, poses, d_map, n_map);
  int64_t launches = 0;
  if ((st = batch_fork(ctx))) return st;
  if ((st = batch_run(ctx, nkf, nullptr, nullptr, d_pose_out, d_success_out, d_ncyl_out,
                      &launches)))
    return st;
  if ((st = batch_join(ctx))) return st;
  ctx->last_launches = launches;
  CK(cudaGetLastError());
  return SLOAM_OK;
}

extern "C" int sloam_keyframes_host(sloam_ctx* ctx, const float* xyzi, int32_t n, int32_t nkf,
                                    const uint8_t* point_labels, const sloam_se3* poses,
                                    const sloam_cylinder* map, int32_t n_map, double* pose_out,
                                    int32_t* success_out, int32_t* ncyl_out) {
  if (!ctx || !xyzi || !point_labels || !poses || nkf < 0 || !pose_out || !success_out ||
      !ncyl_out || n_map <= 0 || !map)
    return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (int g_ = need_weights(ctx)) return g_;
  Dev& d = ctx->d;
  if (n != d.N) return fail(ctx, SLOAM_ERR_ARG, "n must equal img_h * img_w");
  if (ctx->first_scan) return fail(ctx, SLOAM_ERR_ARG, "the context has not seen a first scan");
  if (n_map > d.cap_map) return fail(ctx, SLOAM_ERR_CAPACITY, "map exceeds max_map");
  CK(cudaStreamSynchronize(ctx->st));
  int st = grow_batch(ctx, nkf);
  if (st || (st = grow_front(ctx, nkf, true))) return st;
  if (nkf > ctx->out_cap) {
    if (ctx->d_out_i) cudaFree(ctx->d_out_i);
    if (ctx->d_out_pose) cudaFree(ctx->d_out_pose);
    ctx->d_out_i = nullptr;
    ctx->d_out_pose = nullptr;
    CK(cudaMalloc(&ctx->d_out_i, sizeof(int32_t) * 2 * nkf));
    CK(cudaMalloc(&ctx->d_out_pose, sizeof(double) * 7 * nkf));
    ctx->out_cap = nkf;
  }
  // one map upload shared by every slot (read-only during the batch)
  fill_batch(ctx, nkf, nullptr, nullptr, poses, d.buf_map, n_map);
  int64_t launches = 0;
  if ((st = batch_fork(ctx))) return st;
  CK(cudaMemcpyAsync(d.buf_map, map, sizeof(sloam_cylinder) * n_map, cudaMemcpyHostToDevice,
                     ctx->fe_st));
  if ((st = batch_run(ctx, nkf, xyzi, point_labels, ctx->d_out_pose, ctx->d_out_i,
                      ctx->d_out_i + nkf, &launches)))
    return st;
  if ((st = batch_join(ctx))) return st;
  CK(cudaMemcpyAsync(pose_out, ctx->d_out_pose, sizeof(double) * 7 * nkf, cudaMemcpyDeviceToHost,
                     ctx->st));
  CK(cudaMemcpyAsync(success_out, ctx->d_out_i, sizeof(int32_t) * nkf, cudaMemcpyDeviceToHost,
                     ctx->st));
  CK(cudaMemcpyAsync(ncyl_out, ctx->d_out_i + nkf, sizeof(int32_t) * nkf, cudaMemcpyDeviceToHost,
                     ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  ctx->last_launches = launches;
  return SLOAM_OK;
}

// ------------------------------------------------------ profiling hooks
// Not part of the public header: used by bench.py for per-stage timing and
// the isolated timing of one kernel.  Both replay work on the inputs and
// state left by the previous keyframe call and record CUDA events on the
// context stream.
namespace {
// The profiling hooks replay single-keyframe stages: point the input block's
// cloud and ground views back at the context's own buffers.
int own_views(sloam_ctx* ctx) {
  InPtrs h;
  CK(cudaStreamSynchronize(ctx->st));
  CK(cudaMemcpy(&h, ctx->d.in, sizeof(h), cudaMemcpyDeviceToHost));
  h.tree = ctx->d.tree;
  h.ground = ctx->d.ground;
  h.fe = nullptr;
  h.tflag = nullptr;
  h.gidx = nullptr;
  h.destag = 0;
  CK(cudaMemcpy(ctx->d.in, &h, sizeof(h), cudaMemcpyHostToDevice));
  return SLOAM_OK;
}
}  // namespace

extern "C" int sloam_profile_stages(sloam_ctx* ctx, float* ms, int n) {
  if (!ctx || !ms || n < 4) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  Dev& d = ctx->d;
  if (int st = own_views(ctx)) return st;
  cudaEvent_t ev[5];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0], ctx->st));
  launch_begin(d, -1, -1, -1, -1, -1, ctx->st);
  launch_project(d, ctx->kp, true, ctx->st);
  CK(cudaEventRecord(ev[1], ctx->st));
  launch_trellis(d, ctx->kp, ctx->st);
  CK(cudaEventRecord(ev[2], ctx->st));
  launch_models(d, ctx->kp, true, ctx->st);
  CK(cudaEventRecord(ev[3], ctx->st));
  launch_run(d, ctx->kp, false, false, ctx->st);
  CK(cudaEventRecord(ev[4], ctx->st));
  CK(cudaEventSynchronize(ev[4]));
  for (int i = 0; i < 4; ++i) CK(cudaEventElapsedTime(ms + i, ev[i], ev[i + 1]));
  for (auto& e : ev) cudaEventDestroy(e);
  return SLOAM_OK;
}

// which: 0 = projection kernel (k_project), 1 = the point-cylinder inlier
// counting (inside the work queue: the same as 6), 2 = the proposal network
// on the tensor cores over the last keyframe's samples (cyl_mode 2), 3 = the whole cylinder stage
// (vertex-line fits and the point-level fit of the context's cyl_mode),
// 4 = the Trellis vertex kernel (k_vertex), 5 = the pose solve (k_gn),
// 6 = the cylinder work queue (its ordering and persistent kernels, plain
// RANSAC: cyl_mode >= 1).  All over the last keyframe run on the context.
// Average milliseconds per launch (per stage for 3 and 6) over `reps`.
extern "C" int sloam_time_kernel(sloam_ctx* ctx, int which, int reps, float* avg_ms) {
  if (!ctx || !avg_ms || reps < 1 || which < 0 || which > 6) return SLOAM_ERR_ARG;
  if (which == 1) which = 6;  // the inlier counting runs inside the work queue
  if (which == 2 && (ctx->P.cyl_mode != 2 || !ctx->prop_tc)) return SLOAM_ERR_ARG;
  if ((which == 3 && ctx->P.cyl_mode == 2 && !ctx->prop_tc) ||
      (which == 6 && (ctx->P.cyl_mode < 1 || ctx->kp.K < 1)))
    return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  Dev& d = ctx->d;
  if (int st = own_views(ctx)) return st;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  if (which >= 3) {
    // one event pair per repetition; the queue's inputs are rebuilt before
    // each (it consumes the vertex-line models it refines)
    float total = 0.0f;
    for (int r = 0; r < reps; ++r) {
      if (which == 6) launch_cyl_count_prep(d, ctx->kp, ctx->st);
      CK(cudaEventRecord(a, ctx->st));
      if (which == 3) launch_cylinders(d, ctx->kp, true, ctx->st);
      else if (which == 4) launch_vertex_kernel(d, ctx->kp, ctx->st);
      else if (which == 5) launch_pose_kernel(d, ctx->kp, ctx->st);
      else launch_cyl_queue(d, ctx->kp, nullptr, ctx->st);
      CK(cudaEventRecord(b, ctx->st));
      CK(cudaEventSynchronize(b));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, a, b));
      total += ms;
    }
    *avg_ms = total / reps;
    CK(cudaStreamSynchronize(ctx->st));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return SLOAM_OK;
  }
  // the inlier-counting kernel scores trees still at the vertex-line stage
  CK(cudaEventRecord(a, ctx->st));
  for (int r = 0; r < reps; ++r) {
    if (which == 0) launch_project_kernel(d, ctx->kp, ctx->st);
    else
      prop::launch_prop_infer_trees(d.prop_tc, d.prop_x, &d.cnt->n_lm, ctx->kp.prop_S,
                                    d.prop_cap, d.prop_f, d.prop_out, d.prop_err, ctx->st);
  }
  CK(cudaEventRecord(b, ctx->st));
  CK(cudaEventSynchronize(b));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, a, b));
  *avg_ms = ms / reps;
  if (which == 0) launch_project_rest(d, ctx->kp, true, ctx->st);  // re-arm the pixel keys
  CK(cudaStreamSynchronize(ctx->st));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return SLOAM_OK;
}

// Projection outputs of keyframe k of the last batch call, into host buffers.
extern "C" int sloam_batch_scan_out(sloam_ctx* ctx, int32_t k, sloam_scan_out* out) {
  if (!ctx || !out || k < 0 || k >= ctx->fe_nkf || out->px || out->py) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int n = ctx->d.N;
  const FrontRef& f = ctx->h_refs[k];
  CK(cudaStreamSynchronize(ctx->fe_st));
  CK(cudaStreamSynchronize(ctx->fe_st2));
  int32_t fe[4] = {0, 0, 0, 0};
  CK(cudaMemcpy(fe, f.fe, sizeof(fe), cudaMemcpyDeviceToHost));
  out->n_ground = fe[0];
  if (out->range_image)
    CK(cudaMemcpy(out->range_image, f.range_img, sizeof(float) * n, cudaMemcpyDeviceToHost));
  if (out->mask_out) CK(cudaMemcpy(out->mask_out, f.mask, n, cudaMemcpyDeviceToHost));
  if (out->ground_idx && fe[0] > 0)
    CK(cudaMemcpy(out->ground_idx, f.ground_idx, sizeof(int32_t) * fe[0],
                  cudaMemcpyDeviceToHost));
  if (out->tree_cloud) {
    // the context's own tree-cloud buffer as scratch (rewritten by every
    // keyframe on the context)
    CK(cudaStreamSynchronize(ctx->st));
    launch_tree_out(f, ctx->kp, n, ctx->d.tree, ctx->st);
    CK(cudaMemcpyAsync(out->tree_cloud, ctx->d.tree, sizeof(float4) * n,
                       cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  if (fe[1]) return fail(ctx, SLOAM_ERR_CAPACITY, "batch projection: ground list over max_ground");
  return SLOAM_OK;
}

// Device time of the batch projection of the last batch call: CUDA events
// from the first chunk's projection kernel to the last chunk's compaction.
extern "C" int sloam_frontend_time(sloam_ctx* ctx, float* ms, int32_t* n_chunks,
                                   int32_t* n_keyframes) {
  if (!ctx || !ms) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  // the chunks overlap (a chunk's labels with the next chunk's projection):
  // the span from the first chunk's start to the last chunk's end
  float total = 0.0f;
  if (ctx->fe_chunks > 0) {
    CK(cudaEventSynchronize(ctx->ev_fe[3 * ctx->fe_chunks - 1]));
    CK(cudaEventElapsedTime(&total, ctx->ev_fe[0], ctx->ev_fe[3 * ctx->fe_chunks - 1]));
  }
  *ms = total;
  if (n_chunks) *n_chunks = ctx->fe_chunks;
  if (n_keyframes) *n_keyframes = ctx->fe_nkf;
  return SLOAM_OK;
}

// Learned cylinder proposal weights (FP32, the layout of csrc/proposal.cuh),
// packed once into the bf16 tensor-core operands that every slot reads.
extern "C" int sloam_set_proposal_weights(sloam_ctx* ctx, const float* weights, int32_t n) {
  if (!ctx || !weights || n != prop::kNumParams) return SLOAM_ERR_ARG;
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->st));
  for (auto& s : ctx->extra) CK(cudaStreamSynchronize(s.st));
  if (!ctx->prop_tc) CK(cudaMalloc((void**)&ctx->prop_tc, prop::kTcBytes));
  float* w = nullptr;
  CK(cudaMalloc((void**)&w, sizeof(float) * n));
  cudaError_t e = cudaMemcpyAsync(w, weights, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->st);
  if (e == cudaSuccess) {
    prop::launch_prop_pack(w, ctx->prop_tc, ctx->st);
    e = cudaStreamSynchronize(ctx->st);
  }
  cudaFree(w);
  if (e != cudaSuccess) return fail(ctx, SLOAM_ERR_CUDA, "sloam_set_proposal_weights", e);
  // graphs captured the slots' device state by value
  ctx->d.prop_tc = ctx->prop_tc;
  destroy_graphs(ctx->gx);
  for (auto& s : ctx->extra) {
    s.d.prop_tc = ctx->prop_tc;
    destroy_graphs(s.gx);
  }
  return SLOAM_OK;
}

// Counts of the last single-keyframe call on the context (not part of the
// public header): out = {landmarks, valid cylinders, valid planes, trees that
// fell back to RANSAC (cyl_mode 2), FP64-path projection points}.
extern "C" int sloam_keyframe_stats(const sloam_ctx* ctx, int32_t* out, int n) {
  if (!ctx || !out || n < 5) return SLOAM_ERR_ARG;
  const Counters& c = *ctx->h_cnt;
  out[0] = c.n_lm;
  out[1] = c.n_cyl;
  out[2] = c.n_planes;
  out[3] = c.n_fallback;
  out[4] = c.n_slow_px;
  if (n > 5) out[5] = c.n_fit;
  if (n > 6) out[6] = c.n_fit_pts;
  if (n > 7) out[7] = c.n_bucket;
  if (n > 8) out[8] = c.n_tm + c.n_pm;
  return SLOAM_OK;
}
