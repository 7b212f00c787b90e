// sloam_shim.h — the reference's host-side classes on top of the CUDA C ABI
// (include/sloam_gb300.h), with the reference's names, signatures and
// failure behaviour, so code written against them switches over unchanged
// apart from the stand-in types below.
//
//   reference (file:line)                              here
//   seg::Segmentation  inference.h:55-105              seg::Segmentation
//   Instance           trellis.h:18-65                 Instance
//   Plane              plane.h:21-32                   Plane
//   Cylinder           cylinder.h:25-40                Cylinder
//   ObjectMatch / SloamInput / SloamOutput sloam.h:13-55  same names
//   sloam::sloam       sloam.h:59-105                  sloam::sloam (RunSloam)
//   MapManager         mapManager.h:5-17               MapManager
//   sloam::SLOAMNode   sloamNode.h:30-80               sloam::SLOAMNode (run)
//
// Stand-ins (the reference uses PCL, Eigen, Sophus, OpenCV and ROS types,
// none of which exist here): PointT / CloudT (PCL PointXYZI cloud, with an
// optional per-point label array that replaces the segmentation network's
// output), Vector3 / Vector4, SE3 (unit quaternion + translation), MaskImage
// (cv::Mat of CV_8U), a double stamp instead of ros::Time.
//
// The fitting and the keyframe pipeline run on the GPU through the C ABI;
// there is no CPU path.  Small host methods on the data types (distance,
// project, asPoint) follow the reference's formulas.  CUDA / capacity
// failures throw std::runtime_error (the reference lets third-party
// exceptions escape); algorithmic failures return false like the reference.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sloam_gb300.h"

// ------------------------------------------------------------ stand-ins
struct PointXYZI {
  float x = 0.f, y = 0.f, z = 0.f, intensity = 0.f;
};
static_assert(sizeof(PointXYZI) == 16, "PointXYZI must pack as float4 XYZI");

template <typename P>
struct PointCloud {
  using Ptr = std::shared_ptr<PointCloud<P>>;
  using ConstPtr = std::shared_ptr<const PointCloud<P>>;
  std::vector<P> points;
  uint32_t width = 0, height = 1;   // organised when height > 1
  bool is_dense = true;
  // per-point semantic label (0 other, 1 ground, 255 tree): what the
  // segmentation network would produce; read by seg::Segmentation::run
  std::vector<uint8_t> labels;
  size_t size() const { return points.size(); }
  bool empty() const { return points.empty(); }
  void push_back(const P& p) {
    points.push_back(p);
    width = (uint32_t)points.size();
    height = 1;
  }
  P& operator[](size_t i) { return points[i]; }
  const P& operator[](size_t i) const { return points[i]; }
};

using PointT = PointXYZI;
using CloudT = PointCloud<PointT>;
using Point = PointT;
using Cloud = CloudT;
using Scalar = double;
using VectorType = std::vector<PointT>;
using Slash = VectorType;

struct Vector3 {
  double v[3] = {0, 0, 0};
  Vector3() = default;
  Vector3(double x, double y, double z) : v{x, y, z} {}
  double& operator()(int i) { return v[i]; }
  double operator()(int i) const { return v[i]; }
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
  Vector3 operator+(const Vector3& o) const { return {v[0] + o[0], v[1] + o[1], v[2] + o[2]}; }
  Vector3 operator-(const Vector3& o) const { return {v[0] - o[0], v[1] - o[1], v[2] - o[2]}; }
  Vector3 operator*(double s) const { return {v[0] * s, v[1] * s, v[2] * s}; }
  double dot(const Vector3& o) const { return v[0] * o[0] + v[1] * o[1] + v[2] * o[2]; }
  double norm() const { return std::sqrt(dot(*this)); }
};
inline Vector3 operator*(double s, const Vector3& a) { return a * s; }

struct Vector4 {
  double v[4] = {0, 0, 0, 0};
  double& operator()(int i) { return v[i]; }
  double operator()(int i) const { return v[i]; }
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};

struct Quaternion {
  double w = 1, x = 0, y = 0, z = 0;
};

// Sophus::SE3d stand-in: x -> R x + t, R from a unit quaternion.
class SE3 {
 public:
  SE3() = default;
  SE3(const Quaternion& q, const Vector3& t);
  static SE3 fromC(const sloam_se3& s);
  sloam_se3 toC() const;
  SE3 operator*(const SE3& o) const;
  Vector3 operator*(const Vector3& p) const;
  SE3 inverse() const;
  const Vector3& translation() const { return t_; }
  Vector3& translation() { return t_; }
  Quaternion unit_quaternion() const { return q_; }
  // row-major 3x3
  std::array<double, 9> rotationMatrix() const;

 private:
  Quaternion q_;
  Vector3 t_;
};

struct MaskImage {  // cv::Mat CV_8U stand-in, row-major rows x cols
  int rows = 0, cols = 0;
  std::vector<uint8_t> data;
  uint8_t at(int r, int c) const { return data[(size_t)r * cols + c]; }
};

// ------------------------------------------------------- reference types
struct TreeVertex {  // definitions.h:56-66
  int treeId = 0;
  int beam = 0;
  int prevVertexSize = 0;
  Scalar radius = 0;
  bool isValid = false;
  PointT coords;
  Slash points;
};

struct FeatureModelParams {  // definitions.h:76-106
  int scansPerSweep = 1;
  Scalar minTreeModels = 5;
  Scalar minGroundModels = 36;
  Scalar maxLidarDist = 20;
  Scalar maxGroundLidarDist = 25;
  Scalar minGroundLidarDist = 5;
  bool twoStepOptim = true;
  int groundRadiiBins = 2;
  int groundThetaBins = 18;
  Scalar groundRetainThresh = 0.05;
  Scalar groundMatchThresh = 1.0;
  Scalar roughTreeMatchThresh = 2.5;
  Scalar treeMatchThresh = 0.5;
  Scalar maxTreeRadius = 0.3;
  Scalar maxAxisTheta = 10;
  Scalar maxFocusOutlierDistance = 0.5;
  Scalar AddNewTreeThreshDist = 1.5;
  int featuresPerTree = 20;
  int numGroundFeatures = 5;
  Scalar defaultTreeRadius = 0.2;
};

// sloam_params with the FeatureModelParams fields replaced (the rest kept)
sloam_params to_params(const FeatureModelParams& fm, const sloam_params& base);

template <typename T>
class SemanticObject {  // semanticObject.h:5-19
 public:
  virtual ~SemanticObject() = default;
  virtual Scalar distance(const T& model) const = 0;
  virtual Scalar distance(const PointT& point) const = 0;
  virtual void project(const SE3& tf) = 0;
  T getModel() const { return model; }
  VectorType getFeatures() const { return features; }
  size_t id = 0;
  bool isValid = false;
  VectorType features;
  T model;
};

struct PlaneParameters {  // plane.h:13-18
  Vector4 plane;
  Vector3 centroid;
  double dist = 0;
};

class Plane : public SemanticObject<PlaneParameters> {
 public:
  // plane.cpp:3-17, fitted on the GPU (sloam_fit_plane)
  explicit Plane(const VectorType& points, const FeatureModelParams& fmParams);
  // a plane the pipeline produced (no reference counterpart)
  Plane(const sloam_plane& p, VectorType features);
  Scalar distance(const PlaneParameters& tgt) const override;
  Scalar distance(const PointT& point) const override;
  void project(const SE3& tf) override;
  sloam_plane toC() const;
};

struct CylinderParameters {  // cylinder.h:14-23
  Vector3 root;
  Vector3 ray;
  std::vector<double> radii;
  std::vector<TreeVertex> vertices;
  double radius = 0;
  double lambda = 1;
};

class Cylinder : public SemanticObject<CylinderParameters> {
 public:
  // cylinder.cpp:3-28, fitted on the GPU (sloam_fit_cylinders)
  explicit Cylinder(const std::vector<TreeVertex> vertices, const Plane& gplane,
                    const FeatureModelParams& fmParams);
  // a cylinder the pipeline or a map produced (no reference counterpart)
  Cylinder(const sloam_cylinder& c, VectorType features);
  Scalar distance(const CylinderParameters& model) const override;
  Scalar distance(const PointT& point) const override;
  void project(const SE3& tf) override;
  PointT asPoint(const Scalar height);
  sloam_cylinder toC() const;
};

// ------------------------------------------------------------ segmentation
namespace seg {
class Segmentation {  // inference.h:55-105
 public:
  // modelFilePath and img_d are accepted for signature parity; the labels
  // come from the cloud (no network)
  explicit Segmentation(const std::string modelFilePath, const float fov_up, const float fov_down,
                        const int img_w, const int img_h, const int img_d, bool do_destagger);
  ~Segmentation();
  Segmentation(const Segmentation&) = delete;
  Segmentation& operator=(const Segmentation&) = delete;
  // projection of the labelled cloud; maskImg receives the label of each
  // pixel's nearest point (inference.cpp:80-165 + the network's mask)
  void run(const Cloud::Ptr cloud, MaskImage& maskImg);
  // inference.cpp:230-273: val 1 -> the ground points (compact, point
  // order); val 255 with dense -> the organised tree cloud (NaN elsewhere,
  // destaggered when enabled).  Reads the projection of the last run.
  void maskCloud(const Cloud::Ptr cloud, MaskImage mask, Cloud::Ptr& outCloud, unsigned char val,
                 bool dense = false);

 private:
  void project_(const Cloud::Ptr& cloud, const MaskImage* mask);
  sloam_ctx* ctx_ = nullptr;
  int w_ = 0, h_ = 0;
  std::vector<int32_t> px_, py_, ground_idx_;
  std::vector<float> range_, tree_;
  std::vector<uint8_t> mask_;
  int n_ground_ = 0;
};
}  // namespace seg

// ------------------------------------------------------------------ trellis
class Instance {  // trellis.h:18-65
 public:
  struct Params {
    float beam_cluster_threshold = 0.5f;
    float max_dist_to_centroid = 0.2f;
    int min_vertex_size = 4;
    int min_landmark_size = 5;
    float min_landmark_height = 1.0f;
  };
  explicit Instance();
  ~Instance();
  Instance(const Instance&) = delete;
  Instance& operator=(const Instance&) = delete;
  const Params& params() const { return params_; }
  void set_params(const Params& params) { params_ = params; }
  void reset_tree_id() {}
  // trellis.cpp:134-139 (+ findClusters / findTrees): appends the landmarks
  // of the organised tree_cloud; `cloud` is unused as in the reference
  void computeGraph(const CloudT::Ptr cloud, const CloudT::Ptr tree_cloud,
                    std::vector<std::vector<TreeVertex>>& landmarks);

 private:
  Params params_;
  sloam_ctx* ctx_ = nullptr;
  int w_ = 0, h_ = 0;
};

// -------------------------------------------------------------- sloam core
template <typename T>
struct ObjectMatch {  // sloam.h:13-27
  ObjectMatch(PointT ft, T obj, Scalar d) : feature(ft.x, ft.y, ft.z), object(obj), dist(d) {}
  Vector3 feature;
  T object;
  double dist;
};

struct SloamInput {  // sloam.h:32-45
  SloamInput() : groundCloud(new CloudT()) {}
  SE3 poseEstimate;
  Scalar distance = 0;
  CloudT::Ptr groundCloud;
  std::vector<Cylinder> mapModels;
  std::vector<std::vector<TreeVertex>> landmarks;
};

struct SloamOutput {  // sloam.h:48-55
  std::vector<int> matches;
  std::vector<Cylinder> tm;
  SE3 T_Map_Curr;
  SE3 T_Delta;
};

namespace sloam {
class sloam {  // sloam.h:59-105
 public:
  explicit sloam();
  virtual ~sloam();
  sloam(const sloam&) = delete;
  sloam& operator=(const sloam&) = delete;
  const FeatureModelParams& fmParams() const { return fmParams_; }
  void setFmParams(const FeatureModelParams& fmParams);
  // every parameter of the C ABI at once (no reference counterpart)
  void setParams(const sloam_params& params);
  // sloam.cpp:453-532; models, association, pose and re-projection run on
  // the GPU (sloam_run); the context keeps firstScan_ and prevGPlanes_
  bool RunSloam(SloamInput& in, SloamOutput& out);
  // the planes of the last scan, as the pipeline produced them
  std::vector<Plane> getPrevGroundModel() const { return prevPlanes_; }

 protected:
  sloam_ctx* context() { return ctx_; }
  FeatureModelParams fmParams_;
  sloam_params params_;
  sloam_ctx* ctx_ = nullptr;
  std::vector<Plane> prevPlanes_;
  bool firstScan_ = true;
};
}  // namespace sloam

// ------------------------------------------------------------- map manager
class MapManager {  // mapManager.h:5-17, mapManager.cpp:8-70
 public:
  explicit MapManager(const float searchRadius = 50.f);
  std::vector<Cylinder> getMap();
  // the (up to) 100 map trees nearest to (x, y, 1) of the pose, nearest
  // first (ties by index), that are among the 200 most recently added
  void getSubmap(const SE3& pose, std::vector<Cylinder>& submap);
  void updateMap(std::vector<Cylinder>& obs_tms, const std::vector<int>& matches);
  size_t size() const { return treeModels_.size(); }

 private:
  float sqSearchRadius_;
  std::vector<PointT> landmarks_;
  std::vector<Cylinder> treeModels_;
  std::map<int, int> matchesMap_;
  std::vector<size_t> treeHits_;
};

namespace sloam {
struct NodeParams {  // the ROS parameters SLOAMNode reads (sloamNode.cpp:57-128)
  sloam_params params;
  NodeParams();
};

class SLOAMNode : public sloam {  // sloamNode.h:30-80
 public:
  explicit SLOAMNode(const NodeParams& np);
  ~SLOAMNode() override;
  SLOAMNode(const SLOAMNode&) = delete;
  SLOAMNode& operator=(const SLOAMNode&) = delete;
  using Ptr = std::shared_ptr<SLOAMNode>;
  using ConstPtr = std::shared_ptr<const SLOAMNode>;
  // sloamNode.cpp:186-298: submap query, projection, masks, Trellis,
  // RunSloam (one CUDA graph: sloam_keyframe), map update
  bool run(const SE3 initialGuess, const SE3 prevKeyPose, CloudT::Ptr cloud, double stamp,
           SE3& outPose);
  const std::vector<SE3>& trajectory() const { return trajectory_; }
  MapManager& semanticMap() { return semanticMap_; }

 private:
  MapManager semanticMap_;
  std::vector<SE3> trajectory_;
};
}  // namespace sloam
