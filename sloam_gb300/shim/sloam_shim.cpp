// sloam_shim.cpp — the reference's host classes over the CUDA C ABI (see
// sloam_shim.h for the mapping).
#include "sloam_shim.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <utility>

namespace {

int shim_device() {
  const char* e = std::getenv("SLOAM_GB300_DEVICE");
  return e ? std::atoi(e) : 0;
}

std::string last_error(sloam_ctx* ctx) {
  char buf[512] = {0};
  if (ctx) sloam_last_error(ctx, buf, sizeof(buf));
  return buf;
}

[[noreturn]] void raise(sloam_ctx* ctx, int status, const char* what) {
  throw std::runtime_error(std::string(what) + ": status " + std::to_string(status) + " " +
                           last_error(ctx));
}

sloam_ctx* make_ctx(sloam_params p) {
  p.batch_slots = 1;
  int st = 0;
  sloam_ctx* c = sloam_create(&p, shim_device(), &st);
  if (!c) raise(nullptr, st, "sloam_create");
  return c;
}

sloam_params default_params() {
  sloam_params p{};  // zeroed padding: object_ctx compares parameter blocks bytewise
  sloam_params_default(&p);
  p.batch_slots = 1;
  return p;
}

// One context per thread for the object constructors (Plane, Cylinder),
// re-parameterised when the parameters change.
struct ObjectCtx {
  sloam_ctx* h = nullptr;
  sloam_params p{};
  ~ObjectCtx() {
    if (h) sloam_destroy(h);
  }
};
sloam_ctx* object_ctx(const sloam_params& p) {
  thread_local ObjectCtx oc;
  if (!oc.h) {
    oc.h = make_ctx(p);
    oc.p = p;
  } else if (std::memcmp(&oc.p, &p, sizeof(p)) != 0) {
    sloam_params q = p;
    q.batch_slots = 1;
    const int st = sloam_set_params(oc.h, &q);
    if (st) raise(oc.h, st, "sloam_set_params");
    oc.p = p;
  }
  return oc.h;
}

std::vector<float> pack(const std::vector<PointT>& pts) {
  std::vector<float> v(pts.size() * 4);
  if (!pts.empty()) std::memcpy(v.data(), pts.data(), v.size() * sizeof(float));
  return v;
}

PointT point_of(const float* f) {
  PointT p;
  p.x = f[0];
  p.y = f[1];
  p.z = f[2];
  p.intensity = f[3];
  return p;
}

Vector3 vec(const double* a) { return Vector3(a[0], a[1], a[2]); }

// SoA landmarks of std::vector<std::vector<TreeVertex>> (vertex points as
// the vertex point lists; no component clusters)
struct LandmarkSoA {
  std::vector<int32_t> tree_id, vbeg{0}, vrow, pbeg{0};
  std::vector<float> vxyz, pts;
  std::vector<double> vrad;
  sloam_landmarks c{};
  explicit LandmarkSoA(const std::vector<std::vector<TreeVertex>>& lms) {
    for (const auto& l : lms) {
      tree_id.push_back(l.empty() ? 0 : l[std::min<size_t>(2, l.size() - 1)].treeId);
      for (const auto& v : l) {
        vxyz.insert(vxyz.end(), {v.coords.x, v.coords.y, v.coords.z});
        vrad.push_back(v.radius);
        vrow.push_back(v.beam);
        for (const auto& p : v.points) pts.insert(pts.end(), {p.x, p.y, p.z, p.intensity});
        pbeg.push_back((int32_t)(pts.size() / 4));
      }
      vbeg.push_back((int32_t)vrad.size());
    }
    c.cap_landmarks = c.n_landmarks = (int32_t)tree_id.size();
    c.cap_vertices = c.n_vertices = (int32_t)vrad.size();
    c.cap_points = c.n_points = (int32_t)(pts.size() / 4);
    c.tree_id = tree_id.data();
    c.vertex_begin = vbeg.data();
    c.vertex_xyz = vxyz.data();
    c.vertex_radius = vrad.data();
    c.vertex_row = vrow.data();
    c.point_begin = pbeg.data();
    c.point_xyzi = pts.data();
  }
};

// Output buffers of a models call.
struct ModelsBuf {
  std::vector<sloam_plane> planes;
  std::vector<sloam_cylinder> cyl;
  std::vector<float> feat;
  std::vector<int32_t> inl;
  sloam_models_out c{};
  ModelsBuf(int cap_planes, int cap_cyl, int F)
      : planes(std::max(1, cap_planes)), cyl(std::max(1, cap_cyl)),
        feat((size_t)std::max(1, cap_cyl) * std::max(1, F) * 4), inl(std::max(1, cap_cyl)) {
    c.cap_planes = cap_planes;
    c.cap_cylinders = cap_cyl;
    c.planes = planes.data();
    c.cylinders = cyl.data();
    c.cyl_features = feat.data();
    c.cyl_inliers = inl.data();
  }
  VectorType features(int k, int F) const {
    VectorType v;
    for (int j = 0; j < F; ++j) v.push_back(point_of(&feat[((size_t)k * F + j) * 4]));
    return v;
  }
};

}  // namespace

// ------------------------------------------------------------------ SE3
SE3::SE3(const Quaternion& q, const Vector3& t) : q_(q), t_(t) {
  const double n = std::sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
  q_.w /= n;
  q_.x /= n;
  q_.y /= n;
  q_.z /= n;
}
SE3 SE3::fromC(const sloam_se3& s) {
  return SE3(Quaternion{s.q[3], s.q[0], s.q[1], s.q[2]}, Vector3(s.t[0], s.t[1], s.t[2]));
}
sloam_se3 SE3::toC() const {
  sloam_se3 s;
  s.q[0] = q_.x;
  s.q[1] = q_.y;
  s.q[2] = q_.z;
  s.q[3] = q_.w;
  for (int j = 0; j < 3; ++j) s.t[j] = t_[j];
  return s;
}
std::array<double, 9> SE3::rotationMatrix() const {
  const double w = q_.w, x = q_.x, y = q_.y, z = q_.z;
  return {1 - 2 * (y * y + z * z), 2 * (x * y - w * z),     2 * (x * z + w * y),
          2 * (x * y + w * z),     1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
          2 * (x * z - w * y),     2 * (y * z + w * x),     1 - 2 * (x * x + y * y)};
}
Vector3 SE3::operator*(const Vector3& p) const {
  const auto R = rotationMatrix();
  return Vector3(R[0] * p[0] + R[1] * p[1] + R[2] * p[2] + t_[0],
                 R[3] * p[0] + R[4] * p[1] + R[5] * p[2] + t_[1],
                 R[6] * p[0] + R[7] * p[1] + R[8] * p[2] + t_[2]);
}
SE3 SE3::operator*(const SE3& o) const {
  const Quaternion& a = q_;
  const Quaternion& b = o.q_;
  Quaternion q{a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
               a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
               a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
               a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
  return SE3(q, (*this) * o.t_);
}
SE3 SE3::inverse() const {
  Quaternion qi{q_.w, -q_.x, -q_.y, -q_.z};
  SE3 r(qi, Vector3());
  const Vector3 t = r * t_;
  return SE3(qi, Vector3(-t[0], -t[1], -t[2]));
}

// ----------------------------------------------------------- parameters
sloam_params to_params(const FeatureModelParams& fm, const sloam_params& base) {
  sloam_params p = base;
  p.scans_per_sweep = fm.scansPerSweep;
  p.min_tree_models = fm.minTreeModels;
  p.min_ground_models = fm.minGroundModels;
  p.max_lidar_dist = fm.maxLidarDist;
  p.max_ground_lidar_dist = fm.maxGroundLidarDist;
  p.min_ground_lidar_dist = fm.minGroundLidarDist;
  p.two_step_optim = fm.twoStepOptim ? 1 : 0;
  p.ground_radii_bins = fm.groundRadiiBins;
  p.ground_theta_bins = fm.groundThetaBins;
  p.ground_retain_thresh = fm.groundRetainThresh;
  p.ground_match_thresh = fm.groundMatchThresh;
  p.rough_tree_match_thresh = fm.roughTreeMatchThresh;
  p.tree_match_thresh = fm.treeMatchThresh;
  p.max_tree_radius = fm.maxTreeRadius;
  p.max_axis_theta = fm.maxAxisTheta;
  p.max_focus_outlier_distance = fm.maxFocusOutlierDistance;
  p.add_new_tree_thresh_dist = fm.AddNewTreeThreshDist;
  p.features_per_tree = fm.featuresPerTree;
  p.num_ground_features = fm.numGroundFeatures;
  p.default_tree_radius = fm.defaultTreeRadius;
  return p;
}

// ---------------------------------------------------------------- Plane
Plane::Plane(const VectorType& points, const FeatureModelParams& fmParams) {
  sloam_ctx* ctx = object_ctx(to_params(fmParams, default_params()));
  const std::vector<float> xyzi = pack(points);
  sloam_plane pl{};
  const int st = sloam_fit_plane(ctx, xyzi.data(), (int32_t)points.size(), &pl, nullptr);
  if (st) raise(ctx, st, "sloam_fit_plane");
  features = points;
  isValid = pl.valid != 0;
  if (isValid) {
    features.resize(fmParams.numGroundFeatures);
    for (int j = 0; j < 4; ++j) model.plane[j] = pl.plane[j];
    for (int j = 0; j < 3; ++j) model.centroid[j] = pl.centroid[j];
  }
}
Plane::Plane(const sloam_plane& p, VectorType feats) {
  for (int j = 0; j < 4; ++j) model.plane[j] = p.plane[j];
  for (int j = 0; j < 3; ++j) model.centroid[j] = p.centroid[j];
  features = std::move(feats);
  isValid = p.valid != 0;
}
Scalar Plane::distance(const PlaneParameters& tgt) const {
  return (model.centroid - tgt.centroid).norm();
}
Scalar Plane::distance(const PointT& p) const {
  const double n = std::sqrt(model.plane[0] * model.plane[0] + model.plane[1] * model.plane[1] +
                             model.plane[2] * model.plane[2]);
  return std::fabs(model.plane[0] * p.x + model.plane[1] * p.y + model.plane[2] * p.z +
                   model.plane[3]) /
         n;
}
// plane.cpp:153-170: finite features through tf; plane through tf^-T;
// centroid through tf
void Plane::project(const SE3& tf) {
  for (auto& f : features) {
    if (!std::isfinite(f.x) || !std::isfinite(f.y) || !std::isfinite(f.z)) continue;
    const Vector3 q = tf * Vector3(f.x, f.y, f.z);
    f.x = (float)q[0];
    f.y = (float)q[1];
    f.z = (float)q[2];
  }
  const auto R = tf.rotationMatrix();
  const Vector3 n(model.plane[0], model.plane[1], model.plane[2]);
  const Vector3 rn(R[0] * n[0] + R[1] * n[1] + R[2] * n[2], R[3] * n[0] + R[4] * n[1] + R[5] * n[2],
                   R[6] * n[0] + R[7] * n[1] + R[8] * n[2]);
  model.plane[3] = model.plane[3] - tf.translation().dot(rn);
  for (int j = 0; j < 3; ++j) model.plane[j] = rn[j];
  model.centroid = tf * model.centroid;
}
sloam_plane Plane::toC() const {
  sloam_plane p{};
  for (int j = 0; j < 4; ++j) p.plane[j] = model.plane[j];
  for (int j = 0; j < 3; ++j) p.centroid[j] = model.centroid[j];
  p.bin = -1;
  p.valid = isValid ? 1 : 0;
  return p;
}

// ------------------------------------------------------------- Cylinder
Cylinder::Cylinder(const std::vector<TreeVertex> vertices, const Plane& gplane,
                   const FeatureModelParams& fmParams) {
  const sloam_params p = to_params(fmParams, default_params());
  sloam_ctx* ctx = object_ctx(p);
  LandmarkSoA lm({vertices});
  const sloam_plane pl = gplane.toC();
  ModelsBuf out(1, 1, p.features_per_tree);
  const int st = sloam_fit_cylinders(ctx, &lm.c, &pl, 1, &out.c);
  if (st) raise(ctx, st, "sloam_fit_cylinders");
  model.vertices = vertices;
  for (const auto& v : vertices) model.radii.push_back(v.radius);
  model.lambda = 1;
  isValid = out.c.n_cylinders == 1;
  if (isValid) {
    model.root = vec(out.cyl[0].root);
    model.ray = vec(out.cyl[0].ray);
    model.radius = out.cyl[0].radius;
    id = (size_t)out.cyl[0].id;
    features = out.features(0, p.features_per_tree);
  }
}
Cylinder::Cylinder(const sloam_cylinder& c, VectorType feats) {
  model.root = vec(c.root);
  model.ray = vec(c.ray);
  model.radius = c.radius;
  model.lambda = 1;
  id = (size_t)c.id;
  isValid = c.valid != 0;
  features = std::move(feats);
}
// cylinder.cpp:175-194: mean over z = 0, 3, 6 of the axis-point distance
Scalar Cylinder::distance(const CylinderParameters& tgt) const {
  double s = 0.0;
  for (const double h : {0.0, 3.0, 6.0}) {
    const Vector3 a = model.root + ((h - model.root[2]) / model.ray[2]) * model.ray;
    const Vector3 b = tgt.root + ((h - tgt.root[2]) / tgt.ray[2]) * tgt.ray;
    s += (a - b).norm();
  }
  return s / 3.0;
}
// cylinder.cpp:196-203: distance to the axis minus the radius
Scalar Cylinder::distance(const PointT& point) const {
  const Vector3 p(point.x, point.y, point.z);
  const Vector3 f = model.root + ((p - model.root).dot(model.ray) / model.ray.dot(model.ray)) *
                                     model.ray;
  return (p - f).norm() - model.radius;
}
// cylinder.cpp:205-211: root and root + ray through tf
void Cylinder::project(const SE3& tf) {
  const Vector3 other = model.root + model.ray;
  model.root = tf * model.root;
  model.ray = (tf * other) - model.root;
}
PointT Cylinder::asPoint(const Scalar height) {
  const Vector3 e = model.root + ((height - model.root[2]) / model.ray[2]) * model.ray;
  PointT p;
  p.x = (float)e[0];
  p.y = (float)e[1];
  p.z = 0.f;
  return p;
}
sloam_cylinder Cylinder::toC() const {
  sloam_cylinder c{};
  for (int j = 0; j < 3; ++j) {
    c.root[j] = model.root[j];
    c.ray[j] = model.ray[j];
  }
  c.radius = model.radius;
  c.id = (int32_t)id;
  c.valid = isValid ? 1 : 0;
  return c;
}

// ---------------------------------------------------------- Segmentation
namespace seg {
Segmentation::Segmentation(const std::string, const float fov_up, const float fov_down,
                           const int img_w, const int img_h, const int, bool do_destagger)
    : w_(img_w), h_(img_h) {
  sloam_params p = default_params();
  p.fov_up_deg = fov_up;
  p.fov_down_deg = fov_down;
  p.img_w = img_w;
  p.img_h = img_h;
  p.do_destagger = do_destagger ? 1 : 0;
  p.max_ground = img_w * img_h;
  ctx_ = make_ctx(p);
}
Segmentation::~Segmentation() {
  if (ctx_) sloam_destroy(ctx_);
}
void Segmentation::project_(const Cloud::Ptr& cloud, const MaskImage* mask) {
  const size_t n = (size_t)w_ * h_;
  if (!cloud || cloud->size() != n)
    throw std::invalid_argument("Segmentation: the cloud must hold img_h * img_w points");
  if (!mask && cloud->labels.size() != n)
    throw std::invalid_argument("Segmentation: the cloud carries no per-point labels");
  if (mask && mask->data.size() != n) throw std::invalid_argument("Segmentation: mask size");
  px_.resize(n);
  py_.resize(n);
  range_.resize(n);
  mask_.resize(n);
  ground_idx_.resize(n);
  tree_.resize(n * 4);
  sloam_scan_out so{};
  so.px = px_.data();
  so.py = py_.data();
  so.range_image = range_.data();
  so.mask_out = mask_.data();
  so.ground_idx = ground_idx_.data();
  so.tree_cloud = tree_.data();
  const std::vector<float> xyzi = pack(cloud->points);
  const int st = sloam_project_mask(ctx_, xyzi.data(), (int32_t)n,
                                    mask ? nullptr : cloud->labels.data(),
                                    mask ? mask->data.data() : nullptr, &so);
  if (st) raise(ctx_, st, "sloam_project_mask");
  n_ground_ = so.n_ground;
}
void Segmentation::run(const Cloud::Ptr cloud, MaskImage& maskImg) {
  project_(cloud, nullptr);
  maskImg.rows = h_;
  maskImg.cols = w_;
  maskImg.data = mask_;
}
void Segmentation::maskCloud(const Cloud::Ptr cloud, MaskImage mask, Cloud::Ptr& outCloud,
                             unsigned char val, bool dense) {
  if (mask.data != mask_) project_(cloud, &mask);
  if (!outCloud) outCloud.reset(new CloudT());
  outCloud->points.clear();
  outCloud->labels.clear();
  if (val == 1 && !dense) {
    for (int k = 0; k < n_ground_; ++k) outCloud->points.push_back(cloud->points[ground_idx_[k]]);
    outCloud->width = (uint32_t)outCloud->points.size();
    outCloud->height = 1;
    outCloud->is_dense = true;
  } else if (val == 255 && dense) {
    const size_t n = (size_t)w_ * h_;
    outCloud->points.resize(n);
    for (size_t i = 0; i < n; ++i) outCloud->points[i] = point_of(&tree_[4 * i]);
    outCloud->width = (uint32_t)w_;
    outCloud->height = (uint32_t)h_;
    outCloud->is_dense = false;
  } else {
    throw std::invalid_argument(
        "Segmentation::maskCloud: the path supports val 1 (compact ground) and val 255 "
        "(dense tree cloud)");
  }
}
}  // namespace seg

// -------------------------------------------------------------- Instance
Instance::Instance() = default;
Instance::~Instance() {
  if (ctx_) sloam_destroy(ctx_);
}
void Instance::computeGraph(const CloudT::Ptr, const CloudT::Ptr tree_cloud,
                            std::vector<std::vector<TreeVertex>>& landmarks) {
  if (!tree_cloud || tree_cloud->height <= 1)
    throw std::invalid_argument("Instance::computeGraph: the tree cloud must be organised");
  const int W = (int)tree_cloud->width, H = (int)tree_cloud->height;
  sloam_params p = default_params();
  p.img_w = W;
  p.img_h = H;
  p.max_dist_to_centroid = params_.max_dist_to_centroid;
  p.beam_cluster_threshold = params_.beam_cluster_threshold;
  p.min_vertex_size = params_.min_vertex_size;
  p.min_landmark_size = params_.min_landmark_size;
  p.min_landmark_height = params_.min_landmark_height;
  if (!ctx_ || W != w_ || H != h_) {
    if (ctx_) sloam_destroy(ctx_);
    ctx_ = make_ctx(p);
    w_ = W;
    h_ = H;
  } else {
    const int st = sloam_set_params(ctx_, &p);
    if (st) raise(ctx_, st, "sloam_set_params");
  }
  const int N = W * H, cap_lm = p.max_landmarks, cap_v = cap_lm * p.trellis_max_vertices;
  std::vector<int32_t> tid(cap_lm), vbeg(cap_lm + 1), vrow(cap_v), pbeg(cap_v + 1);
  std::vector<float> vxyz((size_t)cap_v * 3), pts((size_t)N * 4);
  std::vector<double> vrad(cap_v);
  sloam_landmarks lm{};
  lm.cap_landmarks = cap_lm;
  lm.cap_vertices = cap_v;
  lm.cap_points = N;
  lm.tree_id = tid.data();
  lm.vertex_begin = vbeg.data();
  lm.vertex_xyz = vxyz.data();
  lm.vertex_radius = vrad.data();
  lm.vertex_row = vrow.data();
  lm.point_begin = pbeg.data();
  lm.point_xyzi = pts.data();
  const std::vector<float> xyzi = pack(tree_cloud->points);
  const int st = sloam_trellis(ctx_, xyzi.data(), H, W, nullptr, nullptr, &lm);
  if (st) raise(ctx_, st, "sloam_trellis");
  for (int l = 0; l < lm.n_landmarks; ++l) {
    std::vector<TreeVertex> tree;
    for (int v = vbeg[l]; v < vbeg[l + 1]; ++v) {
      TreeVertex tv;
      tv.treeId = tid[l];
      tv.beam = 0;
      tv.prevVertexSize = 0;
      tv.radius = vrad[v];
      tv.isValid = true;
      tv.coords.x = vxyz[3 * v];
      tv.coords.y = vxyz[3 * v + 1];
      tv.coords.z = vxyz[3 * v + 2];
      for (int q = pbeg[v]; q < pbeg[v + 1]; ++q) tv.points.push_back(point_of(&pts[4 * q]));
      tree.push_back(std::move(tv));
    }
    landmarks.push_back(std::move(tree));
  }
}

// ----------------------------------------------------------------- sloam
namespace sloam {
sloam::sloam() : params_(default_params()) { ctx_ = make_ctx(params_); }
sloam::~sloam() {
  if (ctx_) sloam_destroy(ctx_);
}
void sloam::setFmParams(const FeatureModelParams& fmParams) {
  fmParams_ = fmParams;
  params_ = to_params(fmParams, params_);
  const int st = sloam_set_params(ctx_, &params_);
  if (st) raise(ctx_, st, "sloam_set_params");
  firstScan_ = true;
}

void sloam::setParams(const sloam_params& params) {
  params_ = params;
  params_.batch_slots = 1;
  const int st = sloam_set_params(ctx_, &params_);
  if (st) raise(ctx_, st, "sloam_set_params");
  firstScan_ = true;
}

namespace {
// outputs of a run / keyframe call into SloamOutput; returns the reference's
// bool (false on its early-return paths and when the pose did not converge)
bool finish_run(sloam_ctx* ctx, int st, const sloam_run_out& ro, const ModelsBuf& mb,
                const std::vector<int32_t>& matches, int F, SloamOutput& out,
                std::vector<Plane>& prev_planes, bool& first_scan) {
  if (st == SLOAM_ERR_EMPTY_MAP || st == SLOAM_ERR_NO_MODELS) return false;
  if (st != SLOAM_OK && st != SLOAM_ERR_NOT_CONVERGED) raise(ctx, st, "sloam_run");
  out.matches.assign(matches.begin(), matches.begin() + ro.models.n_cylinders);
  out.tm.clear();
  for (int k = 0; k < ro.models.n_cylinders; ++k)
    out.tm.emplace_back(mb.cyl[k], mb.features(k, F));
  out.T_Map_Curr = SE3::fromC(ro.T_Map_Curr);
  out.T_Delta = SE3::fromC(ro.T_Delta);
  prev_planes.clear();
  for (int k = 0; k < ro.models.n_planes; ++k) prev_planes.emplace_back(mb.planes[k], VectorType());
  first_scan = false;
  return st == SLOAM_OK && ro.success;
}
}  // namespace

bool sloam::RunSloam(SloamInput& in, SloamOutput& out) {
  LandmarkSoA lm(in.landmarks);
  std::vector<sloam_cylinder> map;
  for (const auto& m : in.mapModels) map.push_back(m.toC());
  const std::vector<float> ground = pack(in.groundCloud ? in.groundCloud->points : VectorType());
  const int F = params_.features_per_tree;
  ModelsBuf mb(params_.ground_radii_bins * params_.ground_theta_bins,
               std::max(1, lm.c.n_landmarks), F);
  std::vector<int32_t> matches(std::max(1, lm.c.n_landmarks), -1);
  sloam_run_out ro{};
  ro.models = mb.c;
  ro.matches = matches.data();
  const sloam_se3 pose = in.poseEstimate.toC();
  const int st = sloam_run(ctx_, &pose, ground.data(), (int32_t)(ground.size() / 4), &lm.c,
                           map.empty() ? nullptr : map.data(), (int32_t)map.size(), &ro);
  return finish_run(ctx_, st, ro, mb, matches, F, out, prevPlanes_, firstScan_);
}

// ------------------------------------------------------------- SLOAMNode
NodeParams::NodeParams() : params(default_params()) {}

SLOAMNode::SLOAMNode(const NodeParams& np) { setParams(np.params); }
SLOAMNode::~SLOAMNode() = default;

bool SLOAMNode::run(const SE3 initialGuess, const SE3 prevKeyPose, CloudT::Ptr cloud, double,
                    SE3& outPose) {
  const SE3 poseEstimate = prevKeyPose * initialGuess;
  std::vector<Cylinder> mapModels;
  semanticMap_.getSubmap(poseEstimate, mapModels);
  if (!firstScan_ && mapModels.empty()) return false;
  const size_t n = (size_t)params_.img_w * params_.img_h;
  if (!cloud || cloud->size() != n)
    throw std::invalid_argument("SLOAMNode::run: the cloud must hold img_h * img_w points");
  if (cloud->labels.size() != n)
    throw std::invalid_argument("SLOAMNode::run: the cloud carries no per-point labels");
  std::vector<sloam_cylinder> map;
  for (const auto& m : mapModels) map.push_back(m.toC());
  const std::vector<float> xyzi = pack(cloud->points);
  const int F = params_.features_per_tree;
  ModelsBuf mb(params_.ground_radii_bins * params_.ground_theta_bins, params_.max_landmarks, F);
  std::vector<int32_t> matches(params_.max_landmarks, -1);
  sloam_run_out ro{};
  ro.models = mb.c;
  ro.matches = matches.data();
  const sloam_se3 pose = poseEstimate.toC();
  const int st = sloam_keyframe(ctx_, xyzi.data(), (int32_t)n, cloud->labels.data(), nullptr,
                                &pose, map.empty() ? nullptr : map.data(), (int32_t)map.size(),
                                &ro);
  SloamOutput out;
  const bool success = finish_run(ctx_, st, ro, mb, matches, F, out, prevPlanes_, firstScan_);
  semanticMap_.updateMap(out.tm, out.matches);
  if (success) {
    trajectory_.push_back(out.T_Map_Curr);
    outPose = out.T_Map_Curr;
  }
  return success;
}
}  // namespace sloam

// ------------------------------------------------------------ MapManager
MapManager::MapManager(const float searchRadius) : sqSearchRadius_(searchRadius * searchRadius) {}

void MapManager::updateMap(std::vector<Cylinder>& obs_tms, const std::vector<int>& matches) {
  for (size_t i = 0; i < obs_tms.size(); ++i) {
    const Cylinder& tree = obs_tms[i];
    PointT pt;
    pt.x = (float)tree.model.root[0];
    pt.y = (float)tree.model.root[1];
    pt.z = (float)tree.model.root[2];
    if (matches[i] == -1) {
      landmarks_.push_back(pt);
      treeModels_.push_back(tree);
      treeHits_.push_back(1);
    } else {
      const int idx = matchesMap_[matches[i]];
      landmarks_[idx] = pt;
      treeModels_[idx] = tree;
      treeHits_[idx] += 1;
    }
  }
  matchesMap_.clear();
}

std::vector<Cylinder> MapManager::getMap() {
  std::vector<Cylinder> map;
  for (size_t i = 0; i < treeModels_.size(); ++i)
    if (treeHits_[i] > 2) map.push_back(treeModels_[i]);
  return map;
}

void MapManager::getSubmap(const SE3& pose, std::vector<Cylinder>& submap) {
  if (landmarks_.empty()) return;
  const float sx = (float)pose.translation()[0], sy = (float)pose.translation()[1], sz = 1.0f;
  std::vector<std::pair<float, int>> d(landmarks_.size());
  for (size_t i = 0; i < landmarks_.size(); ++i) {
    const float dx = landmarks_[i].x - sx, dy = landmarks_[i].y - sy, dz = landmarks_[i].z - sz;
    d[i] = {dx * dx + dy * dy + dz * dz, (int)i};
  }
  const size_t k = std::min<size_t>(100, d.size());
  std::partial_sort(d.begin(), d.begin() + k, d.end());
  int count = 0;
  const size_t map_size = treeModels_.size();
  for (size_t j = 0; j < k; ++j) {
    const int idx = d[j].second;
    if (map_size - (size_t)idx < 200) {
      matchesMap_[count] = idx;
      submap.push_back(treeModels_[idx]);
      ++count;
    }
  }
}
