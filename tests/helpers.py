"""Shared test helpers: golden fixtures, synthetic scenes, oracle and GPU
wrappers that call the two C ABIs with the same numpy buffers."""
import ctypes as C
import functools
import os

import numpy as np

from oracle import loader as oracle_loader
from sloam_gb300 import capi as A
from sloam_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_aux.npz")

# Tolerances of the fits and of the pose (GPU vs the FP64 oracle)
TOL_AXIS_RAD = 1e-4
TOL_RADIUS_M = 1e-4
TOL_OFFSET_M = 1e-4
TOL_TRANS_M = 1e-5
TOL_ROT_RAD = 1e-6


@functools.lru_cache(None)
def golden():
    return dict(np.load(GOLDEN))


def golden_tree_cloud(seq, t):
    g = golden()
    h, w = g[f"{seq}_{t}_tree_hw"]
    cloud = np.full((h * w, 4), np.nan, np.float32)
    cloud[:, 3] = 0
    cloud[g[f"{seq}_{t}_tree_idx"]] = g[f"{seq}_{t}_tree_xyzi"]
    return cloud, int(h), int(w)


def golden_landmarks(seq, t, resize_points=None):
    """Landmarks as stored by the reference (list of trees of vertex dicts).
    resize_points=5 reproduces core_test.cpp:84 (points resized to 5)."""
    g = golden()
    vb = g[f"{seq}_{t}_lm_vertex_begin"]
    vt = g[f"{seq}_{t}_lm_vertex_tree"]
    vx = g[f"{seq}_{t}_lm_vertex_xyz"]
    vr = g[f"{seq}_{t}_lm_vertex_radius"]
    pb = g[f"{seq}_{t}_lm_point_begin"]
    pts = g[f"{seq}_{t}_lm_points"]
    trees = []
    for l in range(len(vb) - 1):
        tr = []
        for j in range(vb[l], vb[l + 1]):
            p = pts[pb[j]:pb[j + 1]]
            p4 = np.zeros((len(p), 4), np.float32)
            p4[:, :3] = p
            if resize_points is not None:
                q = np.zeros((resize_points, 4), np.float32)
                q[:min(resize_points, len(p4))] = p4[:resize_points]
                p4 = q
            tr.append(dict(tree_id=int(vt[j]), xyz=vx[j], radius=float(vr[j]), row=0, points=p4))
        trees.append(tr)
    return trees


def golden_ground(t):
    return np.ascontiguousarray(golden()[f"still_{t}_ground"])


@functools.lru_cache(None)
def scene(name, seed=0, n_kf=1):
    cfg = {"C1": synth.C1, "C2": synth.C2}[name]
    forest, kfs = synth.scene(cfg, seed=seed, n_kf=n_kf)
    return cfg, forest, kfs


@functools.lru_cache(None)
def c3_scene(counts, seed=0):
    return synth.c3_scene(seed, counts=list(counts))


def oracle():
    return oracle_loader.lib()


# ------------------------------------------------------------- wrappers
def scan_buffers(n, H, W):
    b = dict(px=np.zeros(n, np.int32), py=np.zeros(n, np.int32),
             range_image=np.zeros(H * W, np.float32), mask_out=np.zeros(H * W, np.uint8),
             ground_idx=np.zeros(n, np.int32), tree_cloud=np.zeros((H * W, 4), np.float32))
    s = A.ScanOut()
    s.px = A.ptr(b["px"], C.c_int32)
    s.py = A.ptr(b["py"], C.c_int32)
    s.range_image = A.ptr(b["range_image"], C.c_float)
    s.mask_out = A.ptr(b["mask_out"], C.c_uint8)
    s.ground_idx = A.ptr(b["ground_idx"], C.c_int32)
    s.tree_cloud = A.ptr(b["tree_cloud"], C.c_float)
    return b, s


def oracle_project(P, xyzi, labels=None, mask=None, variant=0):
    H, W = P.img_h, P.img_w
    b, s = scan_buffers(len(xyzi), H, W)
    st = oracle().oracle_project_mask(C.byref(P), A.ptr(xyzi, C.c_float), len(xyzi),
                                      A.ptr(labels, C.c_uint8), A.ptr(mask, C.c_uint8),
                                      variant, C.byref(s))
    assert st == 0
    b["n_ground"] = s.n_ground
    return b


def gpu_project(ctx, xyzi, labels=None, mask=None):
    P = ctx.params
    b, s = scan_buffers(len(xyzi), P.img_h, P.img_w)
    ctx.check(ctx.L.sloam_project_mask(ctx.h, A.ptr(xyzi, C.c_float), len(xyzi),
                                       A.ptr(labels, C.c_uint8), A.ptr(mask, C.c_uint8),
                                       C.byref(s)))
    b["n_ground"] = s.n_ground
    return b


def oracle_trellis(P, cloud, H, W, variant=0, radius_half=0, clusters=True):
    lb = A.LandmarkBuffers(cap_cluster=H * W if clusters else 0)
    labels = np.zeros(H * W, np.uint32)
    nc = C.c_int32()
    st = oracle().oracle_trellis(C.byref(P), A.ptr(cloud, C.c_float), H, W, variant, radius_half,
                                 A.ptr(labels, C.c_uint32), C.byref(nc), C.byref(lb.s))
    assert st == 0
    return lb, labels, nc.value


def gpu_trellis(ctx, cloud, H, W, clusters=True):
    lb = A.LandmarkBuffers(cap_cluster=H * W if clusters else 0)
    labels = np.zeros(H * W, np.uint32)
    nc = C.c_int32()
    ctx.check(ctx.L.sloam_trellis(ctx.h, A.ptr(cloud, C.c_float), H, W,
                                  A.ptr(labels, C.c_uint32), C.byref(nc), C.byref(lb.s)))
    return lb, labels, nc.value


def landmarks_equal_int(a, b):
    """Integer parts of two LandmarkBuffers: ids, vertex counts, rows,
    per-vertex point counts."""
    sa, sb = a.s, b.s
    assert sa.n_landmarks == sb.n_landmarks
    assert sa.n_vertices == sb.n_vertices
    assert sa.n_points == sb.n_points
    nl, nv = sa.n_landmarks, sa.n_vertices
    np.testing.assert_array_equal(a.tree_id[:nl], b.tree_id[:nl])
    np.testing.assert_array_equal(a.vertex_begin[:nl + 1], b.vertex_begin[:nl + 1])
    np.testing.assert_array_equal(a.vertex_row[:nv], b.vertex_row[:nv])
    np.testing.assert_array_equal(a.point_begin[:nv + 1], b.point_begin[:nv + 1])


def landmarks_equal_exact(a, b):
    landmarks_equal_int(a, b)
    nv, npnt = a.s.n_vertices, a.s.n_points
    np.testing.assert_array_equal(a.vertex_xyz[:3 * nv], b.vertex_xyz[:3 * nv])
    np.testing.assert_array_equal(a.vertex_radius[:nv], b.vertex_radius[:nv])
    np.testing.assert_array_equal(a.point_xyzi[:4 * npnt], b.point_xyzi[:4 * npnt])
    if a.s.cluster_begin and b.s.cluster_begin:
        nl = a.s.n_landmarks
        np.testing.assert_array_equal(a.cluster_begin[:nl + 1], b.cluster_begin[:nl + 1])
        k = a.cluster_begin[nl]
        np.testing.assert_array_equal(a.cluster_xyzi[:4 * k], b.cluster_xyzi[:4 * k])


def oracle_models(P, pose, ground, lb):
    s = oracle().oracle_create(C.byref(P))
    mb = A.ModelBuffers(P)
    st = oracle().oracle_compute_models(s, C.byref(pose), A.ptr(ground, C.c_float), len(ground),
                                        C.byref(lb.s), C.byref(mb.s))
    oracle().oracle_destroy(s)
    assert st == 0
    return mb


def gpu_models(ctx, pose, ground, lb):
    mb = A.ModelBuffers(ctx.params)
    ctx.check(ctx.L.sloam_compute_models(ctx.h, C.byref(pose), A.ptr(ground, C.c_float),
                                         len(ground), C.byref(lb.s), C.byref(mb.s)))
    return mb


def angle_between(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    c = abs(np.dot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b))
    return float(np.arccos(min(1.0, c)))


def compare_models(mo, mg, ints_only=False, tol_scale=1.0):
    """Oracle vs GPU models: counts, bins, ids and inlier counts exactly;
    planes and cylinders within the stated tolerances."""
    assert mo.s.n_planes == mg.s.n_planes
    assert mo.s.n_cylinders == mg.s.n_cylinders
    po, pg = mo.plane_array(), mg.plane_array()
    if len(po):
        np.testing.assert_array_equal(po[:, 7], pg[:, 7])  # bins
        if not ints_only:
            for a, b in zip(po, pg):
                assert np.dot(a[:3], b[:3]) > 0  # the same (Eigen's) sign
                assert angle_between(a[:3], b[:3]) < TOL_AXIS_RAD * tol_scale
                # offset where the plane is: the oracle centroid's distance to
                # the GPU plane (d itself grows with the distance of the plane
                # from the map origin: d = -n.c)
                nb = b[:3] / np.linalg.norm(b[:3])
                assert abs(nb @ a[4:7] + b[3] / np.linalg.norm(b[:3])) < TOL_OFFSET_M * tol_scale
                np.testing.assert_allclose(a[4:7], b[4:7], atol=TOL_OFFSET_M * tol_scale)
    co, cg = mo.cyl_array(), mg.cyl_array()
    n = len(co)
    if n:
        np.testing.assert_array_equal(co[:, 7], cg[:, 7])  # tree ids
        np.testing.assert_array_equal(mo.cyl_inliers[:n], mg.cyl_inliers[:n])
        np.testing.assert_array_equal(mo.features(), mg.features())
        if not ints_only:
            for a, b in zip(co, cg):
                assert angle_between(a[3:6], b[3:6]) < TOL_AXIS_RAD * tol_scale, (a, b)
                assert abs(a[6] - b[6]) < TOL_RADIUS_M * tol_scale, (a, b)
                np.testing.assert_allclose(a[0:3], b[0:3], atol=TOL_OFFSET_M * tol_scale)


def rot_angle(q1, q2):
    """Angle (rad) between two unit quaternions (x, y, z, w)."""
    d = abs(float(np.dot(q1 / np.linalg.norm(q1), q2 / np.linalg.norm(q2))))
    return 2.0 * float(np.arccos(min(1.0, d)))
