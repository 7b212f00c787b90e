// internal.h — device state of a context and the kernel launchers of each
// stage.  Everything lives in one device arena sized at context creation
// (nothing is allocated per keyframe).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sloam_gb300.h"

namespace sg {

// Device-side counters and flags of one keyframe.
struct Counters {
  int32_t n_ground;      // ground points (a2)
  int32_t n_comp;        // connected components (a3)
  int32_t n_cand;        // components with > trellis_min_cluster points
  int32_t n_lm;          // landmarks (a4)
  int32_t n_v;           // landmark vertices
  int32_t n_p;           // landmark points
  int32_t n_cluster;     // landmark cluster points
  int32_t n_planes;      // valid ground planes (a7)
  int32_t n_cyl;         // valid cylinders (a6)
  int32_t n_prev;        // planes of the previous scan (state)
  int32_t n_tm;          // tree feature matches
  int32_t n_pm;          // plane feature matches
  int32_t tree_check, ground_check;
  int32_t status;        // SLOAM_* of the pose stage
  int32_t success;
  int32_t overflow;      // bit mask of capacity overflows
  int32_t ransac_fail;
  int32_t n_slow_px;     // projection points that took the FP64 path
  int32_t n_slow_theta;
  int32_t cc_iter_exceeded;
  int32_t n_fallback;    // mode 2: trees that fell back to RANSAC
  int32_t prop_err;      // mode 2: a tensor-core wait gave up
  int32_t queue_err;     // the cylinder work queue: a wait gave up
  int32_t n_fit;         // trees given to the point-level cylinder fit
  int32_t n_fit_pts;     // their points (the work queue's trees)
  int32_t n_bucket;      // tree pixels in the Trellis (component, row) buckets
  int32_t n_wide;        // (component, row) buckets wider than a warp's shared memory
  int32_t pad[4];
};

// The cylinder work queue (cylqueue.cu): the item counter and the shape of
// the current keyframe's queue.
struct QueueCtl {
  int32_t head;    // next item
  int32_t tc;      // counting chunks of the split trees
  int32_t ts;      // LS slices of the split trees (items per LS phase)
  int32_t nq;      // queued trees
  int32_t nsplit;  // of which split over blocks (the first nsplit)
  int32_t phases;  // 1 + LS iterations
};
constexpr int kQueuePhases = 17;  // 1 + at most 16 LS iterations

// Plane and cylinder records used on the device (FP64 models).
struct PlaneD {
  double plane[4];
  double centroid[3];
  int32_t bin;
  int32_t valid;
};
struct CylD {
  double root[3];
  double ray[3];
  double radius;
  int32_t id;
  int32_t valid;
  int32_t inliers;
  int32_t landmark;  // index of the landmark it came from
  int32_t plane;     // nearest plane
  int32_t stage;     // 0 none, 1 vertex line ok (mode 0 model), 2 point fit applied
};

// Per-call inputs, read by the kernels through a device pointer so that a
// captured CUDA graph can be replayed over different input buffers.
// `tree` and `ground` are the organised tree cloud and ground list the later
// stages read: the context's own buffers, or one keyframe's slice of the
// batch projection buffers.  `fe` (batch only) holds that keyframe's
// projection counters {n_ground, overflow, n_slow_px}, copied into the
// counters by the first kernel of the keyframe.
struct InPtrs {
  const float4* xyzi;
  const uint8_t* plabel;
  const uint8_t* mask_in;
  const sloam_cylinder* map;
  const float4* tree;      // organised tree cloud, or null: derived (TreeView)
  const float4* ground;    // ground list, or null: xyzi[gidx[i]] (GroundView)
  const int32_t* fe;
  const uint8_t* tflag;    // per point: its pixel's label is the tree label
  const int32_t* gidx;     // ground list as point indices
  int32_t n_map;
  int32_t destag;          // Ouster destagger applied to the derived tree cloud
};

// The organised tree cloud of maskCloud(..., 255, true) + _destaggerCloud
// (inference.cpp:200-273): materialised, or from the scan and the per-point
// tree flag exactly as the projection's label pass would write it -- x, y, z
// of the point (of point p - 32 on even rows at column >= 32 when
// destaggered) if that point's pixel is a tree pixel, else NaN; the
// intensity of the point itself if its pixel is a tree pixel, else 0.
struct TreeView {
  const float4* tree;
  const float4* xyzi;
  const uint8_t* flag;
  int W;
  int destag;
  __device__ __forceinline__ float4 operator[](int p) const {
    if (tree) return tree[p];
    const float nan = __int_as_float(0x7fc00000);
    const bool f = flag[p] != 0;
    float4 t = f ? xyzi[p] : make_float4(nan, nan, nan, 0.0f);
    if (destag) {
      const int row = p / W, c = p - row * W;
      if ((row & 1) == 0 && c >= 32) {
        const bool fs = flag[p - 32] != 0;
        const float4 s = fs ? xyzi[p - 32] : make_float4(nan, nan, nan, 0.0f);
        t.x = s.x; t.y = s.y; t.z = s.z;
      }
    }
    return t;
  }
};
// The ground list of maskCloud(..., 1): materialised, or as point indices.
struct GroundView {
  const float4* ground;
  const float4* xyzi;
  const int32_t* idx;
  __device__ __forceinline__ float4 operator[](int i) const {
    return ground ? ground[i] : xyzi[idx[i]];
  }
};
__device__ __forceinline__ TreeView tree_view(const InPtrs* in, int W) {
  return TreeView{in->tree, in->xyzi, in->tflag, W, in->destag};
}
__device__ __forceinline__ GroundView ground_view(const InPtrs* in) {
  return GroundView{in->ground, in->xyzi, in->gidx};
}

// One keyframe's projection buffers (a1-a2).  A batch launch reads an array
// of these, one per keyframe, indexed by blockIdx.y.
struct FrontRef {
  const float4* xyzi;
  const uint8_t* plabel;
  const uint8_t* mask_in;
  int32_t* pix;
  unsigned long long* pkey;
  float* range_img;
  uint8_t* mask;
  float4* tree;      // materialised tree cloud (one keyframe on the context)
  uint8_t* tflag;    // per-point tree flag (batch keyframes)
  uint32_t* gbits;
  int32_t* blk;
  int32_t* ground_idx;
  float4* ground;    // materialised ground list, or null (batch keyframes)
  int32_t* fe;  // {n_ground, overflow, n_slow_px, pad}
};

// The vertex-line RANSAC's adaptive iteration bound log(1 - p) /
// log(1 - (c / V)^2) (clamped as PCL clamps it) for every vertex count
// V <= kLineKMax and inlier count c <= V, computed on the host with the
// reference's double expression; larger V evaluate it on the device.
constexpr int kLineKMax = 64;
void build_line_k_table(const sloam_params& p, double* tab);

struct Dev {
  InPtrs* in;          // device copy of the current inputs
  int H, W, N;
  int cap_cand, cap_lm, cap_v, cap_p, cap_ground, cap_map, cap_cluster;
  int n_bins, F, G, K;
  // -- scan (buf_* are the context's own upload buffers)
  float4* buf_xyzi;
  uint8_t* buf_plabel;
  uint8_t* buf_mask_in;
  int32_t* pix;
  unsigned long long* pkey;
  float* range_img;
  uint8_t* mask;
  float4* tree;
  uint32_t* gbits;
  int32_t* blk;        // per-block scratch counts
  int32_t* ground_idx;
  float4* ground;
  float* px_tab;       // [W+1]
  double* line_k;      // [(kLineKMax+1)^2] vertex-line RANSAC iteration bound by (V, inliers)
  float* py_tab;       // [H+1]
  float* tb_tab;       // [Tb+1]
  float* rb_tab;       // [Rb+1]
  float r_lo, r_hi;    // float ground radius window
  // -- connected components
  uint32_t* parent;
  uint32_t* label;
  uint32_t* rank;
  int32_t* comp_size;
  int32_t* comp_cmin;
  int32_t* comp_cmax;
  int32_t* comp_cand;
  // -- Trellis buckets
  int32_t* cand_comp;
  int32_t* rc;         // [cap_cand*H]
  int32_t* roff;       // [cap_cand*H+1]
  int32_t* bucket;     // [N] pixel index per (cand,row) slot, column order
  int32_t* wide_list;  // [cap_cand*H] the wide (cand,row) items of the keyframe
  float4* kept;        // [N] kept vertex points (z order), same offsets
  float4* vmed;        // [cap_cand*H] median (w unused)
  double* vrad;        // [cap_cand*H]
  int32_t* vkept;      // [cap_cand*H] kept count, 0 if not a valid vertex
  int32_t* cand_nv;    // [cap_cand] landmark vertex count (0 = not a landmark)
  int32_t* cand_lm;    // [cap_cand] landmark index or -1
  // -- landmarks (SoA, also filled by uploads)
  int32_t* lm_tree;
  int32_t* lm_vbeg;    // [cap_lm+1]
  float* lm_vxyz;      // [cap_v*3]
  double* lm_vrad;
  int32_t* lm_vrow;
  int32_t* lm_pbeg;    // [cap_v+1]
  float4* lm_pts;      // [cap_p]
  int32_t* lm_cbeg;    // [cap_lm+1]
  float4* lm_cpts;     // [cap_cluster]
  int32_t* lm_vsrc;    // [cap_v] offset of each vertex's kept points in `kept`
  // -- ground bins / planes
  int32_t* bin_of;     // [cap_ground]
  int32_t* bin_cnt;    // [n_bins]
  int32_t* bin_off;    // [n_bins+1]
  unsigned long long* bin_keys;  // [cap_ground]
  PlaneD* plane_all;   // [n_bins]
  float4* plane_feat_all;  // [n_bins*G]
  PlaneD* planes;      // compact [n_bins]
  float4* plane_feat;  // [n_bins*G]
  PlaneD* prev_planes; // [n_bins]
  float4* prev_feat;   // [n_bins*G]
  // -- cylinders
  CylD* cyl_all;       // [cap_lm]
  float4* cyl_feat_all;  // [cap_lm*F]
  unsigned long long* cyl_best;  // [cap_lm] point-fit best (count<<32 | ~h)
  CylD* cyls;          // compact [cap_lm]
  float4* cyl_feat;    // [cap_lm*F]
  // -- map / association / pose
  sloam_cylinder* buf_map;  // [cap_map]
  int32_t* cyl_match;   // [cap_lm] map object matched for the pose (-1)
  int32_t* plane_match; // [n_bins]
  int32_t* match_out;   // [cap_lm] matchModels result
  double* map_pts;      // [cap_map*9] map axis points at z = 0, 3, 6
  float4* map_f;        // [cap_map*3] the same as floats, then max |coordinate|
  float* res_tab;       // [(cap_lm*F + n_bins*G) * 12] residual table of the pose solve
  float2* lm_uv;        // [cap_cluster + cap_p] tree points on the prior axis frame
  float4* hyp;          // [cap_lm * K] circle hypotheses (cu, cv, lo2, hi2)
  int32_t* hyp_cnt;     // [cap_lm * K] inlier counts
  // -- the cylinder work queue (cylqueue.cu)
  QueueCtl* qctl;
  int32_t* q_order;     // [cap_lm] queued trees, largest first
  int32_t* q_off;       // [cap_lm + 1] first chunk of each queued tree
  int32_t* q_soff;      // [cap_lm + 1] first 256-point slice of each queued tree
  int32_t* q_ready;     // [cap_lm] phases the tree has finished
  int32_t* q_done;      // [cap_lm * kQueuePhases] chunks finished per phase
  double* q_st;         // [cap_lm * 16] LS model state
  float* q_sf;          // [cap_lm * 16] its float copies
  float4* q_hyp;        // [cap_lm] the best hypothesis's circle
  float* q_part;        // [q_cap_chunks * 20] slice sums of an LS iteration
  int q_cap_chunks;
  // -- learned proposal (cyl_mode 2); capacities 0 in the other modes
  const unsigned char* prop_tc;  // bf16 network weights (the context's, shared by slots)
  float* prop_x;        // [cap_lm * S][128][3] normalised samples
  float4* prop_f;       // [cap_lm * S] sample mean (xyz), scale (w)
  float* prop_out;      // [cap_lm * S][8] network outputs
  int32_t* pflag;       // [cap_lm] 1: the tree falls back to RANSAC
  int32_t* prop_err;    // &cnt->prop_err
  int prop_cap;         // cap_lm * S (0: mode 0/1)
  double* pose_io;      // [16] in: estimate (q xyzw, t); out: T_Map_Curr, T_Delta
  Counters* cnt;
};

// scalar parameters the kernels need (copied by value into launches)
struct KParams {
  float fov_down_abs, fov;
  int img_w, img_h, do_destagger;
  float cc_thr;
  int min_cluster, min_beam, min_vertices, max_vertices;
  float max_d_centroid;
  int Rb, Tb;
  double retain_num;
  int G, F;
  double max_lidar_dist, min_tree_height_sq, root_plane_max_dist;
  double max_tree_radius, max_axis_theta, default_tree_radius;
  double line_thr;
  int line_max_iter;
  double line_prob;
  uint64_t seed;
  int cyl_mode, K, ls_iters;
  int prop_S;          // learned proposals per tree (mode 2)
  float prop_ratio;    // fallback below this inlier ratio
  float tau, max_hyp_r;
  double tree_match_thresh, plane_match_thresh, add_new_tree_thresh;
  double min_tree_models, min_ground_models, min_planes;
  int two_step;
  int gn_iters;
  int pose_lm, lm_iters;  // trust-region LM instead of fixed GN iterations
  double huber;
  int cc_iter_limit;      // retries of one connected-components union
  int q_chunk, q_tile, q_blocks;  // cylinder work queue shape (tuned)
};

// Default retry limit of a connected-components union (a CAS loop that
// contention can repeat; a union normally takes one or two rounds).
constexpr int kCCIterLimitDefault = 1 << 20;

KParams make_kparams(const sloam_params& p);

// ---------------------------------------------------------------- stages
// Every launcher enqueues on `st` and returns the number of kernels launched.
int launch_project(const Dev& d, const KParams& kp, bool point_labels, cudaStream_t st);
// a1-a2 for keyframes [kf0, kf0 + nkf) of refs (device array), one launch per kernel
// A chunk of batch keyframes: the projection kernel, then (on another
// stream, after it) the label and compaction kernels.
int launch_project_batch_points(const Dev& d, const KParams& kp, const FrontRef* refs,
                                int kf0, int nkf, bool point_labels, cudaStream_t st);
int launch_project_batch_labels(const Dev& d, const FrontRef* refs, int kf0, int nkf,
                                bool point_labels, cudaStream_t st);
size_t front_gbits_words(int N);
int launch_tree_out(const FrontRef& f, const KParams& kp, int N, float4* out, cudaStream_t st);
int front_blocks(int N);
int launch_trellis(const Dev& d, const KParams& kp, cudaStream_t st);
void init_trellis_attributes();
int launch_models(const Dev& d, const KParams& kp, bool from_trellis, cudaStream_t st);
int launch_run(const Dev& d, const KParams& kp, bool first_scan, bool update_state,
               cudaStream_t st, bool map_prepped = false);
// k_map_prep alone (a keyframe graph runs it beside the models)
int launch_map_prep(const Dev& d, cudaStream_t st);
// point-level cylinder fit of the trees `only` marks (all eligible: NULL) by
// the persistent work queue; cylqueue.cu
int launch_cyl_queue(const Dev& d, const KParams& kp, const int32_t* only, cudaStream_t st);
bool queue_shape_valid(int chunk_points, int hyp_tile);
int launch_vertex_kernel(const Dev& d, const KParams& kp, cudaStream_t st);
int launch_pose_kernel(const Dev& d, const KParams& kp, cudaStream_t st);
void init_queue_attributes();
int launch_fit_cylinder_points(const Dev& d, const KParams& kp, bool from_trellis,
                               cudaStream_t st);
// a6 alone: cylinders of the landmarks against the planes already in d.planes
int launch_cylinders(const Dev& d, const KParams& kp, bool from_trellis, cudaStream_t st);
// The two halves of the model stage a keyframe graph runs side by side: the
// ground planes (needs the ground list) and the cylinder fits (needs the
// landmarks), then the plane gates and the cylinder list (needs both).
int launch_planes(const Dev& d, const KParams& kp, cudaStream_t st);
int launch_cylinder_fits(const Dev& d, const KParams& kp, bool from_trellis, cudaStream_t st);
int launch_cylinder_close(const Dev& d, const KParams& kp, cudaStream_t st);
// Plane(points) of the n points of the ground view into plane_all[0]
int launch_plane_points(const Dev& d, const KParams& kp, int n, cudaStream_t st);

// single kernels, for isolated timing (profiling hooks)
int launch_project_kernel(const Dev& d, const KParams& kp, cudaStream_t st);
// the projection stage after k_project (labels, tree cloud, ground list, key re-arm)
int launch_project_rest(const Dev& d, const KParams& kp, bool point_labels, cudaStream_t st);
int launch_cyl_fit_kernel(const Dev& d, const KParams& kp, cudaStream_t st);
int launch_cyl_count_prep(const Dev& d, const KParams& kp, cudaStream_t st);

// per-call counter reset: counts >= 0 are set, -1 left to the pipeline
int launch_begin(const Dev& d, int n_ground, int n_lm, int n_v, int n_p, int n_cluster,
                 cudaStream_t st);
void init_kernel_attributes();

// learned cylinder proposal (proposal.cu): bf16 tensor-core operands from the
// FP32 weights (prop::kTcBytes), and inference over n normalised 128-point
// samples into out[n][8] (mode 0 tensor cores, 1 SIMT reference)
namespace prop {
int launch_prop_pack(const float* d_w, unsigned char* d_tcw, cudaStream_t st);
int launch_prop_infer(const unsigned char* d_tcw, const float* d_x, int n, float* d_out,
                      int* d_err, int mode, cudaStream_t st);
// tensor-core inference over (*d_n_trees) groups of per_tree samples (at
// most cap samples); groups whose frame scale (d_frames[first].w) is 0 skip
int launch_prop_infer_trees(const unsigned char* d_tcw, const float* d_x, const int* d_n_trees,
                            int per_tree, int cap, const float4* d_frames, float* d_out,
                            int* d_err, cudaStream_t st);
void init_attributes();
}  // namespace prop

// Device view of a map manager (mapmgr.cu): the map, hit counts, scratch,
// the last submap and its map indices; state = {n, n_submap, overflow}.
struct MapMgrDev {
  int cap, k, recent;
  sloam_cylinder* models;  // [cap]
  int32_t* hits;           // [cap]
  float* dist;             // [cap] squared distances of the last query
  sloam_cylinder* sub;     // [k]
  int32_t* sub_idx;        // [k] map index of each submap entry
  int32_t* slot;           // [k] rank -> map index scratch
  int32_t* state;          // [4]
};
// submap query at (x, y); with d_in, also points the keyframe input block's
// map at the submap (map, n_map written on the device)
int launch_mm_submap(const MapMgrDev& m, double x, double y, InPtrs* d_in, cudaStream_t st);
// map update with the keyframe's cylinders and matches (reads its status)
int launch_mm_update(const MapMgrDev& m, const Dev& d, int first, cudaStream_t st);
const MapMgrDev& mapmgr_dev(const sloam_mapmgr* mm);
int mapmgr_device(const sloam_mapmgr* mm);

// host-built tables (context.cu)
void build_px_table(const sloam_params& p, float* tab);
void build_py_table(const sloam_params& p, float* tab);
void build_ground_tables(const sloam_params& p, float* tb, float* rb, float* r_lo,
                         float* r_hi);

}  // namespace sg
