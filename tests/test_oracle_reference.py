"""The oracle pinned against the reference's own tests and fixtures.

- Trellis known answers: sloam/src/tests/aux/{still,moving}_tree_t{0,1}.pcd
  -> {still,moving}_landmarks_t{0,1} (converted by tests/golden/make_golden.py).
- plane_test.cpp:57-96, cylinder_test.cpp:69-126, core_test.cpp:128-193 as
  property tests on the oracle.
- Philox4x32-10 known-answer vectors (Random123 kat_vectors).
"""
import ctypes as C

import numpy as np
import pytest

from sloam_gb300 import capi as A
from tests import helpers as H


@pytest.mark.parametrize("seq", ["still", "moving"])
@pytest.mark.parametrize("t", ["t0", "t1"])
@pytest.mark.parametrize("variant", [0, 1])
def test_trellis_matches_reference_fixture(seq, t, variant):
    cloud, h, w = H.golden_tree_cloud(seq, t)
    P = A.default_params()
    lb, labels, ncomp = H.oracle_trellis(P, cloud, h, w, variant=variant, radius_half=1)
    ref = H.golden_landmarks(seq, t)
    trees = lb.to_trees()
    assert len(trees) == len(ref)
    for tr, rt in zip(trees, ref):
        assert len(tr) == len(rt)
        for v, rv in zip(tr, rt):
            assert v["tree_id"] == rv["tree_id"]
            # the PCD stores 8 significant digits, the archive 10
            np.testing.assert_allclose(v["xyz"], rv["xyz"], atol=2e-6, rtol=0)
            assert abs(v["radius"] - rv["radius"]) < 2e-6
            assert v["points"].shape == rv["points"].shape
            np.testing.assert_allclose(v["points"][:, :3], rv["points"][:, :3], atol=2e-6, rtol=0)


def test_trellis_component_labels_raster_order():
    cloud, h, w = H.golden_tree_cloud("still", "t0")
    P = A.default_params()
    lb, labels, ncomp = H.oracle_trellis(P, cloud, h, w)
    valid = labels != 0xFFFFFFFF
    assert np.array_equal(valid, np.isfinite(cloud[:, 0]))
    # first pixel of every component appears in increasing label order
    first = {}
    for i in np.nonzero(valid)[0]:
        first.setdefault(int(labels[i]), int(i))
    order = [first[k] for k in range(ncomp)]
    assert order == sorted(order)


def plane_params(G):
    # plane_test.cpp:34-58
    return A.default_params(max_lidar_dist=15.0, max_ground_lidar_dist=30.0,
                            min_ground_lidar_dist=0.0, ground_radii_bins=1,
                            ground_theta_bins=18, ground_match_thresh=2.0,
                            ground_retain_thresh=0.1, num_ground_features=G,
                            max_tree_radius=0.3, max_axis_theta=10,
                            tree_match_thresh=1.0, add_new_tree_thresh_dist=2.0,
                            features_per_tree=2, default_tree_radius=0.1)


def oracle_plane(P, pts):
    pts = np.asarray([[*p, 0] for p in pts], np.float32)
    pl = A.Plane()
    H.oracle().oracle_plane(C.byref(P), A.ptr(pts, C.c_float), len(pts), C.byref(pl), None)
    return pl


def test_plane_initializes():  # plane_test.cpp:63-72
    pl = oracle_plane(plane_params(1), [(0, 0, 0), (0, 1, 0), (1, 0, 0)])
    assert pl.valid


def test_plane_distance_to_feature():  # plane_test.cpp:74-86
    pl = oracle_plane(plane_params(1), [(0, 0, 0), (0, 1, 0), (1, 0, 0)])
    d = H.oracle().oracle_plane_distance_point(C.byref(pl), (C.c_float * 3)(0, 0, 0))
    assert abs(d) < 0.1


def test_plane_translate_model():  # plane_test.cpp:88-96
    pl = oracle_plane(plane_params(1), [(0, 0, 0), (0, 1, 0), (1, 0, 0)])
    c2 = pl.centroid[2]
    tf = A.SE3.from_qt((0, 0, 0, 1), (0, 0, 1))
    H.oracle().oracle_plane_project(C.byref(pl), C.byref(tf))
    assert pl.centroid[2] == c2 + 1


def cylinder_params():
    # cylinder_test.cpp:47-67
    return A.default_params(max_lidar_dist=30.0, max_ground_lidar_dist=30.0,
                            min_ground_lidar_dist=0.0, ground_radii_bins=1,
                            ground_theta_bins=1, ground_match_thresh=2.0,
                            ground_retain_thresh=0.1, max_tree_radius=0.3, max_axis_theta=10,
                            tree_match_thresh=1.0, add_new_tree_thresh_dist=2.0,
                            features_per_tree=2, num_ground_features=3,
                            default_tree_radius=0.1)


def oracle_cylinders():
    P = cylinder_params()
    plane = oracle_plane(P, [(0, 0, 0), (0, 1, 0), (1, 0, 0), (1, 1, 0)])
    lb = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t0"))
    out = []
    for l in range(lb.s.n_landmarks):
        c = A.Cylinder()
        feat = np.zeros((P.features_per_tree, 4), np.float32)
        H.oracle().oracle_cylinder(C.byref(P), C.byref(lb.s), l, C.byref(plane), C.byref(c),
                                   A.ptr(feat, C.c_float), None)
        if c.valid:
            out.append((c, feat))
    return out


def test_cylinder_initializes_and_some_valid():  # cylinder_test.cpp:69-77
    assert len(oracle_cylinders()) > 0


def test_cylinder_distance_to_model():  # cylinder_test.cpp:79-93
    c, _ = oracle_cylinders()[0]
    assert H.oracle().oracle_cylinder_distance_model(C.byref(c), C.byref(c)) == 0.0


def test_cylinder_distance_to_feature():  # cylinder_test.cpp:95-108
    c, feat = oracle_cylinders()[0]
    d = H.oracle().oracle_cylinder_distance_point(C.byref(c), A.ptr(np.ascontiguousarray(feat[0, :3]), C.c_float))
    assert abs(d) < 0.1


def test_cylinder_translate_model():  # cylinder_test.cpp:110-126
    c, _ = oracle_cylinders()[0]
    r0 = c.root[0]
    tf = A.SE3.from_qt((0, 0, 0, 1), (1, 0, 0))
    H.oracle().oracle_cylinder_project(C.byref(c), C.byref(tf))
    assert c.root[0] == r0 + 1


def core_params(two_step):
    # core_test.cpp:94-119 (twoStepOptim and the model minima are left
    # uninitialised there; both optimiser paths are exercised here)
    return A.default_params(max_lidar_dist=15.0, max_ground_lidar_dist=30.0,
                            min_ground_lidar_dist=0.0, ground_radii_bins=1,
                            ground_theta_bins=18, ground_match_thresh=2.0,
                            ground_retain_thresh=0.05, max_tree_radius=0.3, max_axis_theta=10,
                            tree_match_thresh=1.0, add_new_tree_thresh_dist=2.0,
                            features_per_tree=2, num_ground_features=60,
                            default_tree_radius=0.1, two_step_optim=two_step,
                            min_tree_models=0, min_ground_models=0, min_planes=0)


def oracle_run_pair(P):
    L = H.oracle()
    s = L.oracle_create(C.byref(P))
    lm0 = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t0", resize_points=5))
    lm1 = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t1", resize_points=5))
    g0, g1 = H.golden_ground("t0"), H.golden_ground("t1")
    I = A.SE3.identity()
    r0 = A.RunBuffers(P)
    st0 = L.oracle_run(s, C.byref(I), A.ptr(g0, C.c_float), len(g0), C.byref(lm0.s), None, 0,
                       C.byref(r0.s))
    r0.refresh()
    m = A.cylinders_from_array(r0.m.cyl_array())
    r1 = A.RunBuffers(P)
    st1 = L.oracle_run(s, C.byref(I), A.ptr(g1, C.c_float), len(g1), C.byref(lm1.s), m,
                       r0.s.models.n_cylinders, C.byref(r1.s))
    r1.refresh()
    L.oracle_destroy(s)
    return st0, r0, st1, r1


@pytest.mark.parametrize("two_step", [0, 1])
def test_core_first_second_scan_success_association(two_step):
    st0, r0, st1, r1 = oracle_run_pair(core_params(two_step))
    assert st0 == 0 and r0.s.models.n_cylinders > 0 and r0.s.models.n_planes > 0  # FirstScan
    assert st1 == 0 and r1.s.success                                              # SLOAMSucess
    assert r1.s.models.n_cylinders > 0
    assert (r1.matches[:r1.s.models.n_cylinders] != -1).any()                     # ObjectAssociation
    # PoseOptimization: |T_Delta.t| < 0.1 (identity on the two-step path)
    assert np.linalg.norm(np.array(r1.s.T_Delta.t[:])) < 0.1 or two_step == 0


def test_core_pose_stays_near_identity_joint():
    # core_test.cpp:177 bounds |T_Delta.t| by 0.1 m; tests/test_plane_sign.py
    # holds the same bound for both pose solvers
    st0, r0, st1, r1 = oracle_run_pair(core_params(0))
    assert np.linalg.norm(np.array(r1.s.T_Map_Curr.t[:])) < 0.1


# Random123 kat_vectors, philox4x32 10 rounds
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    out = (C.c_uint32 * 4)()
    H.oracle().oracle_philox((key[1] << 32) | key[0], (C.c_uint32 * 4)(*ctr), out)
    assert tuple(out) == expect


def test_projection_contract_vs_libm_and_ties():
    """The correctly rounded contract and the literal host-libm expression
    place at most a handful of points differently (glibc's atan2f is within
    one ulp but not correctly rounded)."""
    cfg, forest, kfs = H.scene("C2")
    P = H.synth.preset_params(cfg)
    kf = kfs[0]
    a = H.oracle_project(P, kf.xyzi, labels=kf.labels, variant=0)
    b = H.oracle_project(P, kf.xyzi, labels=kf.labels, variant=1)
    diff = int(((a["px"] != b["px"]) | (a["py"] != b["py"])).sum())
    assert diff <= 10
    # nearest point wins: every pixel's range is the minimum over its points
    pix = a["py"] * P.img_w + a["px"]
    r = np.sqrt((kf.xyzi[:, :3].astype(np.float64) ** 2).sum(1)).astype(np.float32)
    finite = np.isfinite(r)
    best = np.full(P.img_w * P.img_h, np.inf, np.float32)
    np.minimum.at(best, pix[finite], r[finite])
    has = np.isfinite(best)
    np.testing.assert_allclose(a["range_image"][has], best[has], rtol=1e-6)


def test_oracle_run_empty_map_and_no_models():
    P = core_params(1)
    L = H.oracle()
    s = L.oracle_create(C.byref(P))
    lm0 = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t0", resize_points=5))
    g0 = H.golden_ground("t0")
    I = A.SE3.identity()
    r = A.RunBuffers(P)
    assert L.oracle_run(s, C.byref(I), A.ptr(g0, C.c_float), len(g0), C.byref(lm0.s), None, 0,
                        C.byref(r.s)) == 0
    r = A.RunBuffers(P)
    assert L.oracle_run(s, C.byref(I), A.ptr(g0, C.c_float), len(g0), C.byref(lm0.s), None, 0,
                        C.byref(r.s)) == A.SLOAM_ERR_EMPTY_MAP
    empty = A.LandmarkBuffers.from_trees([])
    m = A.cylinders_from_array(np.array([[0, 0, 0, 0, 0, 1, 0.2, 0]]))
    assert L.oracle_run(s, C.byref(I), A.ptr(g0, C.c_float), len(g0), C.byref(empty.s), m, 1,
                        C.byref(r.s)) == A.SLOAM_ERR_NO_MODELS
    L.oracle_destroy(s)
