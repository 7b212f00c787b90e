/*
 * sloam_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * C API of the CPU oracle: a std-only C++17 restatement of the SLOAM keyframe
 * path of KumarRobotics/sloam (inference.cpp, trellis.cpp, plane.cpp,
 * cylinder.cpp, sloam.cpp).  Only the tests, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it, as the checker and
 * as the timed CPU baseline.  The product path never links it.
 *
 * Parity is pinned against the reference's own test fixtures
 * (sloam/src/tests/aux: the {still,moving}_tree_t{0,1}.pcd clouds and their
 * {still,moving}_landmarks_t{0,1} Trellis outputs) and
 * the property tests of plane_test.cpp / cylinder_test.cpp / core_test.cpp.
 */
#ifndef SLOAM_ORACLE_H
#define SLOAM_ORACLE_H

#include "../include/sloam_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic variants of the projection.
 *  ORACLE_CONTRACT: correctly-rounded atan2f/asinf, nearest point wins a
 *                   pixel with ties to the lowest point index (the contract
 *                   the GPU kernels are bit-exact against).
 *  ORACLE_LIBM:     the reference expression literally (std::atan2(float),
 *                   std::asin(float), std::sort of the ranges) - used to
 *                   count how many pixels the host libm would place
 *                   differently. */
#define ORACLE_CONTRACT 0
#define ORACLE_LIBM     1

int oracle_project_mask(const sloam_params* p, const float* xyzi, int32_t n,
                        const uint8_t* point_labels, const uint8_t* mask_image,
                        int variant, sloam_scan_out* out);

/* Trellis.  sort_variant: ORACLE_CONTRACT orders vertex points by
 * (z, y, x, column); ORACLE_LIBM runs std::sort x, y, z like trellis.cpp.
 * radius_half: 1 stores 0.5*|first-last| (the convention of the reference's
 * stored fixtures), 0 the current formula |first-last| (trellis.cpp:96-99).
 * out->cluster_* (may be NULL): every point of each landmark's CC cluster
 * in raster order, for the point-level cylinder fit. */
int oracle_trellis(const sloam_params* p, const float* tree_cloud, int32_t H,
                   int32_t W, int sort_variant, int radius_half,
                   uint32_t* cc_labels, int32_t* n_components,
                   sloam_landmarks* out);

typedef struct oracle_state oracle_state;
oracle_state* oracle_create(const sloam_params* p);
void          oracle_destroy(oracle_state* s);
void          oracle_set_params(oracle_state* s, const sloam_params* p);
void          oracle_reset(oracle_state* s);

/* computeModels (sloam.cpp:388-436).  Without lm->cluster_* the point-level
 * cylinder fit uses the landmark's vertex points. */
int oracle_compute_models(oracle_state* s, const sloam_se3* pose,
                          const float* ground_xyzi, int32_t n_ground,
                          const sloam_landmarks* lm, sloam_models_out* out);

/* RunSloam (sloam.cpp:453-532). */
int oracle_run(oracle_state* s, const sloam_se3* pose, const float* ground_xyzi,
               int32_t n_ground, const sloam_landmarks* lm,
               const sloam_cylinder* map, int32_t n_map, sloam_run_out* out);

/* Whole keyframe: projection + mask, Trellis, RunSloam. */
int oracle_keyframe(oracle_state* s, const float* xyzi, int32_t n,
                    const uint8_t* point_labels, const uint8_t* mask_image,
                    const sloam_se3* pose, const sloam_cylinder* map,
                    int32_t n_map, sloam_run_out* out);

/* Single objects (Plane::Plane, Cylinder::Cylinder and their methods) */
int    oracle_plane(const sloam_params* p, const float* xyzi, int32_t n,
                    sloam_plane* out, float* features);
int    oracle_cylinder(const sloam_params* p, const sloam_landmarks* lm,
                       int32_t landmark, const sloam_plane* plane,
                       sloam_cylinder* out, float* features, int32_t* inliers);
double oracle_cylinder_distance_model(const sloam_cylinder* self,
                                      const sloam_cylinder* tgt);
double oracle_cylinder_distance_point(const sloam_cylinder* self,
                                      const float* xyz);
void   oracle_cylinder_project(sloam_cylinder* c, const sloam_se3* tf);
double oracle_plane_distance_point(const sloam_plane* self, const float* xyz);
void   oracle_plane_project(sloam_plane* pl, const sloam_se3* tf);

/* Philox4x32-10 block, for tests of the RNG contract. */
void oracle_philox(uint64_t key, const uint32_t ctr[4], uint32_t out[4]);

/* Third column of U of Eigen 3.3.7's JacobiSVD of the 3 x n matrix `a`
 * (row-major: x row, y row, z row), the plane normal with Eigen's sign. */
void oracle_eigen_svd_u3(const double* a, int32_t n, double u3[3]);

#ifdef __cplusplus
}
#endif
#endif
