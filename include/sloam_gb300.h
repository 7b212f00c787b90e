/*
 * sloam_gb300.h — C ABI of the GB300 (sm_103a) SLOAM keyframe hot path.
 *
 * Every entry point is plain C: POD structs, raw pointers and sizes, an int
 * status (0 = OK).  No C++ exceptions and no torch types cross this boundary.
 * The caller owns every host buffer; a context owns its device buffers and one
 * CUDA stream.  A context is thread-compatible: use one context per thread.
 *
 * Which reference interface each entry point replaces is stated beside it
 * (paths are relative to the KumarRobotics/sloam repository).
 */
#ifndef SLOAM_GB300_H
#define SLOAM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define SLOAM_OK                 0
#define SLOAM_ERR_ARG            1  /* bad argument / size                          */
#define SLOAM_ERR_CUDA           2  /* a CUDA runtime call failed                   */
#define SLOAM_ERR_TIMEOUT        3  /* a bounded device-side wait gave up           */
#define SLOAM_ERR_EMPTY_MAP      4  /* sloam.cpp:476-480  not first scan, empty map */
#define SLOAM_ERR_NO_MODELS      5  /* sloam.cpp:482-486  no ground or landmarks    */
#define SLOAM_ERR_NOT_CONVERGED  6  /* sloam.cpp:241     pose solve failed          */
#define SLOAM_ERR_CAPACITY       7  /* an output or scratch capacity was exceeded   */
#define SLOAM_ERR_NO_DEVICE      8  /* no CUDA device / kernels not loadable        */

/* ------------------------------------------------------------ parameters */
/* One POD mirroring FeatureModelParams (include/helpers/definitions.h:76-104),
 * Instance::Params (include/segmentation/trellis.h:31-40), the Segmentation
 * constructor arguments (inference.h:57-58) and every constant the reference
 * hard-codes on the path, made explicit.  sloam_params_default() fills the
 * values of params/sloam.yaml and sloamNode.cpp:57-128. */
typedef struct sloam_params {
  /* FeatureModelParams */
  int32_t scans_per_sweep;
  double  min_tree_models;          /* min_tree_models            (5)     */
  double  min_ground_models;        /* min_ground_models          (36)    */
  double  max_lidar_dist;           /* max_lidar_dist             (20)    */
  double  max_ground_lidar_dist;    /* max_ground_dist            (25)    */
  double  min_ground_lidar_dist;    /* min_ground_dist            (5)     */
  int32_t two_step_optim;           /* two_step_optim             (1)     */
  int32_t ground_radii_bins;        /* ground_radii_bins          (2)     */
  int32_t ground_theta_bins;        /* ground_theta_bins          (18)    */
  double  ground_retain_thresh;     /* ground_retain_thresh       (0.05)  */
  double  ground_match_thresh;      /* ground_match_thresh        (1.0)   */
  double  rough_tree_match_thresh;  /* rough_tree_match_thresh    (2.5)   */
  double  tree_match_thresh;        /* tree_match_thresh          (0.5)   */
  double  max_tree_radius;          /* sloamNode.cpp:104          (0.3)   */
  double  max_axis_theta;           /* sloamNode.cpp:105          (10 deg)*/
  double  max_focus_outlier_distance;/* sloamNode.cpp:106         (0.5)   */
  double  add_new_tree_thresh_dist; /* add_new_tree_thresh_dist   (1.5)   */
  int32_t features_per_tree;        /* features_per_tree          (20)    */
  int32_t num_ground_features;      /* num_ground_features        (5)     */
  double  default_tree_radius;      /* default_tree_radius        (0.2)   */
  /* minPlanes_ of sloam.cpp:11.  The reference reads it from an
   * uninitialised struct; here it is explicit (default 0.1 * bins). */
  double  min_planes;

  /* Instance::Params */
  float   beam_cluster_threshold;   /* (0.5, unused on the path)          */
  float   max_dist_to_centroid;     /* (0.2) trellis.cpp:90               */
  int32_t min_vertex_size;          /* (4,   unused on the path)          */
  int32_t min_landmark_size;        /* (5,   unused on the path)          */
  float   min_landmark_height;      /* (1.0, unused on the path)          */

  /* Segmentation (range-image projection) */
  float   fov_up_deg;               /* seg_lidar_fov  (+22.5)             */
  float   fov_down_deg;             /* -seg_lidar_fov (-22.5)             */
  int32_t img_w;                    /* seg_lidar_w    (2048)              */
  int32_t img_h;                    /* seg_lidar_h    (64)                */
  int32_t do_destagger;             /* do_destagger   (1)                 */

  /* constants hard-coded in the reference, explicit here */
  float   cc_dist_threshold;        /* trellis.cpp:23         1.0 m       */
  int32_t trellis_min_cluster;      /* trellis.cpp:109        > 80 pts    */
  int32_t trellis_min_beam_points;  /* trellis.cpp:119        > 3 pts     */
  int32_t trellis_min_vertices;     /* trellis.cpp:124        > 16        */
  int32_t trellis_max_vertices;     /* trellis.cpp:125-126    56          */
  double  line_ransac_thresh;       /* cylinder.cpp:122       0.25 m      */
  int32_t line_ransac_max_iter;     /* PCL SACSegmentation default 50     */
  double  line_ransac_probability;  /* PCL SACSegmentation default 0.99   */
  double  min_tree_height_sq;       /* cylinder.cpp:109       1.5 m^2     */
  double  root_plane_max_dist;      /* cylinder.cpp:48        2.0 m       */
  double  plane_match_thresh;       /* sloam.cpp:490          1.0 m       */
  double  huber_delta;              /* sloam.cpp:69,130,181   0.1         */

  /* extensions of this implementation (no reference counterpart) */
  uint64_t seed;                    /* RANSAC counter-based RNG key       */
  int32_t cyl_mode;                 /* 0 = vertex-line RANSAC (reference) ;
                                       1 = + point-level cylinder RANSAC ;
                                       2 = + learned proposals, RANSAC as
                                           fallback                       */
  int32_t cyl_hypotheses;           /* K hypotheses per tree (mode 1)     */
  float   cyl_inlier_thresh;        /* tau, metres (mode 1)               */
  int32_t cyl_ls_iters;             /* LS refinement iterations (mode 1)  */
  float   cyl_max_hyp_radius;       /* reject circle hypotheses above     */
  int32_t gn_iters;                 /* Gauss-Newton iterations (pose)     */
  int32_t max_landmarks;            /* context capacity: trees per scan   */
  int32_t max_map;                  /* context capacity: submap cylinders */
  int32_t max_ground;               /* context capacity: ground points    */
  int32_t batch_slots;              /* keyframes of a batch in flight at
                                       once (each slot owns buffers, a
                                       stream and a captured graph)       */
  int32_t prop_samples;             /* mode 2: network proposals per tree
                                       (128-point samples, 1..8)      (8) */
  float   prop_min_inlier_ratio;    /* mode 2: best proposal's inliers /
                                       tree points below this -> RANSAC
                                       fallback for the tree        (0.6) */
  int32_t pose_solver;              /* 0 = Gauss-Newton, gn_iters fixed
                                       iterations (0) ; 1 = trust-region
                                       Levenberg-Marquardt with the solver
                                       settings the reference gives Ceres
                                       (sloam.cpp:91-97: at most
                                       lm_max_iters iterations, default
                                       trust-region options)              */
  int32_t lm_max_iters;             /* max_num_iterations (sloam.cpp:92) (50) */
  /* shape of the point-level cylinder fit's work queue (modes 1 and 2):
     chosen per GPU and workload by sloam_gb300/autotune.py            */
  int32_t cyl_chunk_points;         /* points per work item: 256, 512 or
                                       1024                          (256) */
  int32_t cyl_hyp_tile;             /* hypotheses staged per pass: 64, 128,
                                       256, 512 or 1024              (256) */
  int32_t cyl_queue_blocks;         /* persistent blocks (0: 76)           */
} sloam_params;

void sloam_params_default(sloam_params* p);

/* --------------------------------------------------------- common types */
/* SE(3) as a unit quaternion (x, y, z, w) and a translation. */
typedef struct sloam_se3 {
  double q[4];
  double t[3];
} sloam_se3;

/* Landmarks in Trellis form: the output of Instance::computeGraph
 * (trellis.cpp:134-139), std::vector<std::vector<TreeVertex>> flattened to
 * SoA.  Vertex v of landmark l is v in [vertex_begin[l], vertex_begin[l+1]),
 * bottom beam first; its kept points are [point_begin[v], point_begin[v+1])
 * in z order (x, y, z, intensity).  The caller sets the cap_* fields and the
 * pointers; the callee sets n_*.  vertex_row is the range-image row of the
 * vertex (the reference stores beam = 0). */
typedef struct sloam_landmarks {
  int32_t  cap_landmarks, cap_vertices, cap_points;
  int32_t  n_landmarks, n_vertices, n_points;
  int32_t* tree_id;        /* [cap_landmarks]    CC label of the tree     */
  int32_t* vertex_begin;   /* [cap_landmarks+1]                           */
  float*   vertex_xyz;     /* [cap_vertices*3]   per-axis median          */
  double*  vertex_radius;  /* [cap_vertices]                              */
  int32_t* vertex_row;     /* [cap_vertices]                              */
  int32_t* point_begin;    /* [cap_vertices+1]                            */
  float*   point_xyzi;     /* [cap_points*4]                              */
  /* optional: every point of each landmark's connected component in raster
   * order (cluster_begin[cap_landmarks+1]), used by the point-level
   * cylinder fit; NULL pointers = not requested / not provided */
  int32_t  cap_cluster, n_cluster;
  int32_t* cluster_begin;
  float*   cluster_xyzi;   /* [cap_cluster*4]                             */
} sloam_landmarks;

/* Cylinder model (CylinderParameters, cylinder.h:8-17) */
typedef struct sloam_cylinder {
  double  root[3];
  double  ray[3];
  double  radius;
  int32_t id;              /* tree id (vertex[2].treeId)                  */
  int32_t valid;
} sloam_cylinder;

/* Plane model (PlaneParameters, plane.h:13-18) */
typedef struct sloam_plane {
  double  plane[4];        /* n (unit), d                                 */
  double  centroid[3];
  int32_t bin;             /* r_bin * theta_bins + t_bin                  */
  int32_t valid;
} sloam_plane;

/* ------------------------------------------------------------- context */
typedef struct sloam_ctx sloam_ctx;

/* Creates a context on `device`.  Replaces the construction of
 * seg::Segmentation (inference.cpp:5-19), Instance (trellis.cpp:13) and
 * sloam::sloam (sloam.cpp:6-12) state owned by SLOAMNode (sloamNode.cpp:57-118).
 * Returns NULL and sets *status on failure. */
sloam_ctx* sloam_create(const sloam_params* params, int device, int* status);
void       sloam_destroy(sloam_ctx* ctx);
/* Copies the last error message (NUL-terminated) into buf. */
int        sloam_last_error(const sloam_ctx* ctx, char* buf, size_t n);
/* Resets the per-sequence state (firstScan_, prevGPlanes_; sloam.cpp:9-10). */
int        sloam_reset(sloam_ctx* ctx);
/* Replaces the parameters (sloam::sloam::setFmParams, sloam.h:77). */
int        sloam_set_params(sloam_ctx* ctx, const sloam_params* params);

/* ------------------------------------------ a1/a2: projection + masking */
/* Segmentation::_doProjection (inference.cpp:80-165) followed by
 * Segmentation::maskCloud (inference.cpp:230-273) for val = 1 (ground list)
 * and val = 255, dense (organised tree cloud, destaggered per
 * inference.cpp:200-228).  Input is n = H*W points, packed x,y,z,intensity.
 * Labels come either as a per-pixel mask image (the network output, codes
 * 0/1/255, `mask_image` non-NULL) or as per-point labels (`point_labels`
 * non-NULL): the mask of a pixel is then the label of the point that wins the
 * pixel (the nearest).  Any output pointer may be NULL.
 *   px, py       [n]     pixel of each point (proj_xs/proj_ys)
 *   range_image  [H*W]   range of the winning point, 0 where empty
 *   mask_out     [H*W]   mask used
 *   ground_idx   [n]     indices of ground points, point order; *n_ground
 *   tree_cloud   [H*W*4] organised tree cloud, NaN xyz where not tree   */
typedef struct sloam_scan_out {
  int32_t* px;
  int32_t* py;
  float*   range_image;
  uint8_t* mask_out;
  int32_t* ground_idx;
  int32_t  n_ground;
  float*   tree_cloud;
} sloam_scan_out;

int sloam_project_mask(sloam_ctx* ctx, const float* xyzi, int32_t n,
                       const uint8_t* point_labels, const uint8_t* mask_image,
                       sloam_scan_out* out);

/* ------------------------------------------------ a3-a5: Trellis       */
/* Instance::computeGraph (trellis.cpp:134-139): organised connected
 * components (trellis.cpp:15-43) + per-beam vertices (trellis.cpp:45-132).
 * tree_cloud is the organised H*W cloud (x,y,z,i; NaN = no tree).
 * cc_labels [H*W] (may be NULL) receives the component label of each pixel
 * (0xFFFFFFFF where not finite); *n_components the number of components. */
int sloam_trellis(sloam_ctx* ctx, const float* tree_cloud, int32_t H, int32_t W,
                  uint32_t* cc_labels, int32_t* n_components,
                  sloam_landmarks* out);

/* --------------------------------------- a6-a8: ground planes, cylinders */
/* sloam::computeModels (sloam.cpp:388-436): ground binning
 * (sloam.cpp:330-386), Plane (plane.cpp:3-17,96-128) with the angle/height
 * gates, then per landmark the nearest plane and Cylinder
 * (cylinder.cpp:3-173).  Outputs the valid planes and valid cylinders in
 * reference order; cyl_features [cap_cyl*features_per_tree*4] receives the
 * F features of each valid cylinder (may be NULL). */
typedef struct sloam_models_out {
  int32_t         cap_planes, cap_cylinders;
  int32_t         n_planes, n_cylinders;
  sloam_plane*    planes;
  sloam_cylinder* cylinders;
  float*          cyl_features;
  int32_t*        cyl_inliers;    /* [cap_cyl] best RANSAC inlier count (mode 1:
                                     point cylinder, else vertex line) */
} sloam_models_out;

int sloam_compute_models(sloam_ctx* ctx, const sloam_se3* pose_estimate,
                         const float* ground_xyzi, int32_t n_ground,
                         const sloam_landmarks* landmarks,
                         sloam_models_out* out);

/* Plane::Plane(points, fmParams) (plane.cpp:3-17, computeModel :96-128):
 * the plane of all n points (float centroid, smallest-eigenvalue normal
 * with the sign Eigen 3.3's JacobiSVD gives it, as the reference's
 * plane.cpp:113-115 does), valid iff n >= num_ground_features (no gates;
 * those belong to computeModels).  features [num_ground_features*4]
 * receives the first points (may be NULL).  n <= max_ground. */
int sloam_fit_plane(sloam_ctx* ctx, const float* xyzi, int32_t n, sloam_plane* out,
                    float* features);

/* Cylinder::Cylinder(vertices, gplane, fmParams) (cylinder.cpp:3-28) for
 * every landmark, each against the nearest of the given planes
 * (sloam.cpp:414-435 with the planes supplied instead of binned from a
 * ground cloud).  out->planes echoes the given planes; out->cylinders holds
 * the valid cylinders in landmark order.  n_planes <= radii_bins*theta_bins. */
int sloam_fit_cylinders(sloam_ctx* ctx, const sloam_landmarks* landmarks,
                        const sloam_plane* planes, int32_t n_planes,
                        sloam_models_out* out);

/* --------------------------------------------- a9-a11: RunSloam        */
/* sloam::sloam::RunSloam (sloam.cpp:453-532): computeModels, first-scan
 * logic, matchFeatures (sloam.cpp:257-296), OptimizePose /
 * TwoStepOptimizePose (sloam.cpp:33-255), projectModels (sloam.cpp:438-451)
 * and matchModels (sloam.cpp:298-328).  Keeps firstScan_ / prevGPlanes_ in
 * the context like the reference object.
 *   map       [n_map]  submap cylinders (SloamInput::mapModels, map frame)
 *   out->matches [cap_cylinders]  index into map or -1 (SloamOutput::matches)
 *   out->models.cylinders          SloamOutput::tm (map frame)
 * Returns SLOAM_OK on success; SLOAM_ERR_EMPTY_MAP / SLOAM_ERR_NO_MODELS /
 * SLOAM_ERR_NOT_CONVERGED where the reference returns false. */
typedef struct sloam_run_out {
  sloam_models_out models;       /* tm (projected) + current planes        */
  int32_t*  matches;             /* [models.cap_cylinders]                 */
  sloam_se3 T_Map_Curr;
  sloam_se3 T_Delta;
  int32_t   success;
  int32_t   first_scan;
  int32_t   n_tree_matches;      /* feature matches (residuals), trees     */
  int32_t   n_plane_matches;     /* feature matches (residuals), planes    */
  int32_t   tree_check, ground_check;
} sloam_run_out;

int sloam_run(sloam_ctx* ctx, const sloam_se3* pose_estimate,
              const float* ground_xyzi, int32_t n_ground,
              const sloam_landmarks* landmarks,
              const sloam_cylinder* map, int32_t n_map,
              sloam_run_out* out);

/* ---------------------------------------------- whole keyframe          */
/* SLOAMNode::run (sloamNode.cpp:186-282) minus the ROS publishing, the
 * segmentation network and the map manager: projection + masking, Trellis,
 * RunSloam on one scan, all on the device in one CUDA graph.  pose_estimate
 * is prevKeyPose * initialGuess; map is the submap the map manager supplies. */
int sloam_keyframe(sloam_ctx* ctx, const float* xyzi, int32_t n,
                   const uint8_t* point_labels, const uint8_t* mask_image,
                   const sloam_se3* pose_estimate,
                   const sloam_cylinder* map, int32_t n_map,
                   sloam_run_out* out);

/* Device-resident batch for throughput.  d_xyzi / d_point_labels / d_map
 * and the three outputs are device pointers; pose_estimates is a host array
 * of nkf poses.  The nkf scans (n points each, back to back) are processed
 * as independent non-first keyframes against the same submap and the
 * context's previous-scan planes; the context state is not advanced (the
 * context must have seen a first scan).  Per keyframe: T_Map_Curr (7
 * doubles: q xyzw, t), the success flag and the number of valid cylinders. */
int sloam_keyframes_device(sloam_ctx* ctx, const float* d_xyzi, int32_t n,
                           int32_t nkf, const uint8_t* d_point_labels,
                           const sloam_se3* pose_estimates,
                           const sloam_cylinder* d_map, int32_t n_map,
                           double* d_pose_out, int32_t* d_success_out,
                           int32_t* d_ncyl_out);

/* Host-buffer batch: the same as sloam_keyframes_device with every pointer a
 * host pointer (xyzi [nkf*n*4], point_labels [nkf*n], map [n_map]; pinned
 * host memory lets the copies overlap the compute).  Keyframes are spread
 * over the context's batch_slots (buffers + stream + graph each), their
 * host->device copies interleaved with the work of the other slots;
 * pose_out [nkf*7], success_out [nkf], ncyl_out [nkf] are host arrays,
 * complete when the call returns.  Each keyframe is SLOAMNode::run's work
 * (sloamNode.cpp:186-282) for one scan. */
int sloam_keyframes_host(sloam_ctx* ctx, const float* xyzi, int32_t n, int32_t nkf,
                         const uint8_t* point_labels, const sloam_se3* pose_estimates,
                         const sloam_cylinder* map, int32_t n_map, double* pose_out,
                         int32_t* success_out, int32_t* ncyl_out);

/* Projection outputs of keyframe k of the last batch call (the outputs of
 * Segmentation::maskCloud for that scan, inference.cpp:200-273), into host
 * buffers as sloam_project_mask gives them: range_image, mask_out,
 * ground_idx (+ n_ground) and tree_cloud (derived from the batch's
 * per-point tree flags and the scan, which must still be in place for a
 * device batch).  px and py are not kept for batch keyframes and must be
 * NULL.  Valid until the next batch call. */
int sloam_batch_scan_out(sloam_ctx* ctx, int32_t k, sloam_scan_out* out);

/* Device time of the last batch call's projection (CUDA events from the
 * first chunk's projection kernel to the last chunk's ground compaction; a
 * chunk's label kernels overlap the next chunk's projection), the number of
 * chunks and of keyframes they covered. */
int sloam_frontend_time(sloam_ctx* ctx, float* ms, int32_t* n_chunks, int32_t* n_keyframes);

/* Input ingestion (pcl::fromROSMsg at inputNode.cpp:247 and the XYZI
 * packing of inference.cpp:374-379, on the device): n points of a
 * sensor message with point_step bytes per point and little-endian fields
 * at the given byte offsets (x, y, z float32; intensity per
 * intensity_type) packed into float4 XYZI (d_xyzi [n*4]) on `stream`
 * (a cudaStream_t, NULL = default).  Device pointers; the caller owns both
 * buffers.  The layout of a sensor_msgs/PointCloud2 (e.g. an Ouster cloud:
 * point_step 48, x 0, y 4, z 8, intensity 16 float32). */
#define SLOAM_FIELD_NONE    0
#define SLOAM_FIELD_FLOAT32 1
#define SLOAM_FIELD_UINT16  2
#define SLOAM_FIELD_UINT8   3
int sloam_pack_points(const void* d_points, int32_t n, int32_t point_step, int32_t off_x,
                      int32_t off_y, int32_t off_z, int32_t off_i, int32_t intensity_type,
                      float* d_xyzi, void* stream);

/* Weights of the learned cylinder proposal (cyl_mode 2; no reference
 * counterpart): n = 75399 FP32 values of the point-set network
 * (shared MLP 3-64-128-256, max-pool, head 256-128-7, row-major W[in][out]
 * then bias, layer by layer), trained by sloam_gb300/proposal.py; stored
 * as bf16 for the tensor cores.  A context in cyl_mode 2 refuses keyframes
 * until weights are set. */
int sloam_set_proposal_weights(sloam_ctx* ctx, const float* weights, int32_t n);

/* Training and evaluation of the proposal network (no reference
 * counterpart; sloam_gb300/proposal.py drives them).  They run on the
 * current device with their own temporaries.
 * sloam_prop_num_params: 75399.
 * sloam_prop_sample: n synthetic trunk clusters, Philox-keyed by (seed,
 *   first_id + i): d_points [n*128*3] centred and scale-normalised,
 *   d_targets [n*8] (axis, centre xy, log(r/s), s, r).
 * sloam_prop_train: `steps` Adam steps (lr, betas 0.9/0.999, eps 1e-8) of
 *   `batch` fresh clusters each (samples of seed ^ 0x5a5a5a5a, ids from
 *   first_id), from `init` (NULL: seeded uniform init); weights_out
 *   [75399], loss_out [steps] mean losses (may be NULL).
 * sloam_prop_grad: one step's mean gradient grad_out [75399] (and the n
 *   per-cluster losses, loss_out may be NULL) of `weights` on device
 *   samples, without the update.
 * sloam_prop_infer: network outputs d_out [n*8] for device samples; mode 0
 *   the tensor-core kernel, 1 the SIMT kernel of the same arithmetic. */
int sloam_prop_num_params(void);
int sloam_prop_sample(uint64_t seed, int64_t first_id, int32_t n, float* d_points,
                      float* d_targets);
int sloam_prop_train(const float* init, int32_t steps, int32_t batch, float lr, uint64_t seed,
                     int64_t first_id, float* weights_out, float* loss_out);
int sloam_prop_grad(const float* weights, const float* d_points, const float* d_targets,
                    int32_t n, float* grad_out, float* loss_out);
int sloam_prop_infer(const float* weights, const float* d_points, int32_t n, float* d_out,
                     int32_t mode);

/* Projection + masking that allocates nothing (no reference counterpart: it
 * exists for callers that cannot call cudaMalloc, such as plugins inside a
 * process whose allocator owns the GPU or real-time loops that forbid
 * allocation after start-up).  The same kernels as sloam_project_mask;
 * every intermediate buffer lives in a file-scope __device__ array of about
 * 4.2 MB that each GPU loading the library holds until exit, sized for at
 * most 131072 points (H*W) and width 4096 - larger scans are rejected with
 * SLOAM_ERR_CAPACITY.  All data pointers are device pointers: d_xyzi [n*4],
 * d_point_labels [n] or d_mask_image [H*W], and the outputs d_ground_idx
 * [n], d_n_ground [1], d_tree_cloud [H*W*4] and, optionally (NULL skips),
 * d_pix [n] (py*W + px), d_range_image [H*W], d_mask_out [H*W].  `stream`
 * is a cudaStream_t (NULL = legacy default stream); results are ready when
 * the stream reaches them.  The first call in each CUDA context (a device's
 * primary context, or one the caller made current) looks up the array's
 * address in that context.  Every call copies its boundary tables and input
 * pointers from host memory, so the call cannot be captured into a CUDA
 * graph (issue it on a stream that is not capturing).  All calls of a
 * context share the one array: calls that overlap on the GPU (other
 * streams, other threads) race.  Host code must treat the array only
 * through this entry point. */
int sloam_project_mask_noalloc(const sloam_params* params, const float* d_xyzi, int32_t n,
                               const uint8_t* d_point_labels, const uint8_t* d_mask_image,
                               int32_t* d_pix, float* d_range_image, uint8_t* d_mask_out,
                               int32_t* d_ground_idx, int32_t* d_n_ground,
                               float* d_tree_cloud, void* stream);

/* ---- Map manager on the GPU (MapManager, mapManager.h:7-10) ------------
 * The landmark map, its hit counts, the submap query and the update stay
 * in device memory.  getSubmap (mapManager.cpp:41-68): the k nearest map
 * roots to (x, y, 1) - squared distances summed in double and rounded to
 * float, ties to the lower map index; the reference's k is 100 (:54) - of
 * which those among the `recent` most recently added (200, :60) form the
 * submap, in distance order.  updateMap (mapManager.cpp:8-28): each
 * cylinder in order; no match appends it with one hit, a match overwrites
 * the matched entry and adds a hit. */
typedef struct sloam_mapmgr sloam_mapmgr;

/* MapManager::MapManager (mapManager.cpp:3): an empty map of up to
 * `capacity` landmarks on `device`. */
int sloam_mapmgr_create(int32_t device, int32_t capacity, int32_t k, int32_t recent,
                        sloam_mapmgr** out);
int sloam_mapmgr_destroy(sloam_mapmgr* mm);
/* Map size, size of the last submap, and 1 when an append found the map
 * full (the cylinder was dropped). */
int sloam_mapmgr_size(sloam_mapmgr* mm, int32_t* n, int32_t* n_submap, int32_t* overflow);
/* MapManager::getMap (mapManager.cpp:30-39), with the hit counts: up to
 * `cap` entries into host arrays; *n = the map size. */
int sloam_mapmgr_read(sloam_mapmgr* mm, sloam_cylinder* models, int32_t* hits, int32_t cap,
                      int32_t* n);
/* Replaces the map by n host entries. */
int sloam_mapmgr_load(sloam_mapmgr* mm, const sloam_cylinder* models, const int32_t* hits,
                      int32_t n);
/* MapManager::getSubmap at (x, y): the submap into host arrays (its map
 * indices too, NULL skips), *n_out = its size. */
int sloam_mapmgr_submap(sloam_mapmgr* mm, double x, double y, sloam_cylinder* out,
                        int32_t* map_index, int32_t cap, int32_t* n_out);
/* One keyframe of SLOAMNode::runSLOAMNode with the device map
 * (sloamNode.cpp:197-236): getSubmap at the pose's (x, y), RunSloam on it
 * (as sloam_keyframe, with the submap as the map), then updateMap with the
 * keyframe's cylinders and matches when the status is SLOAM_OK or
 * SLOAM_ERR_NOT_CONVERGED.  A later keyframe whose submap is empty returns
 * SLOAM_ERR_EMPTY_MAP and leaves the map unchanged (sloamNode.cpp:199). */
int sloam_keyframe_mapped(sloam_ctx* ctx, sloam_mapmgr* mm, const float* xyzi, int32_t n,
                          const uint8_t* point_labels, const uint8_t* mask_image,
                          const sloam_se3* pose, sloam_run_out* out);

/* Returns the number of kernels launched by the last call (for accounting). */
int64_t sloam_last_launch_count(const sloam_ctx* ctx);

/* The CUDA stream the context runs on (as void*). */
void* sloam_stream(sloam_ctx* ctx);

/* Retry limit of one connected-components union (no reference counterpart:
 * the union is a compare-and-swap loop that contention can repeat).  When a
 * union runs out of rounds the kernel records it and returns, and the call
 * ends with SLOAM_ERR_TIMEOUT and "connected-components union loop hit its
 * iteration limit"; the context stays usable.  limit < 0 restores the
 * default (2^20); 0 makes every union that is needed give up at once
 * (used to test that path).  Drops the captured keyframe graphs. */
int sloam_set_cc_iter_limit(sloam_ctx* ctx, int32_t limit);

#ifdef __cplusplus
}
#endif
#endif /* SLOAM_GB300_H */
