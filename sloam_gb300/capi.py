"""ctypes mirrors of the structs in include/sloam_gb300.h.

The layouts here must match the C header field for field; a CPU test checks
sizeof() of each struct against the library's own `sloam_abi_sizes` export.
"""
import ctypes as C

import numpy as np

SLOAM_OK = 0
SLOAM_ERR_ARG = 1
SLOAM_ERR_CUDA = 2
SLOAM_ERR_TIMEOUT = 3
SLOAM_ERR_EMPTY_MAP = 4
SLOAM_ERR_NO_MODELS = 5
SLOAM_ERR_NOT_CONVERGED = 6
SLOAM_ERR_CAPACITY = 7
SLOAM_ERR_NO_DEVICE = 8

STATUS_NAMES = {
    0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_TIMEOUT", 4: "ERR_EMPTY_MAP",
    5: "ERR_NO_MODELS", 6: "ERR_NOT_CONVERGED", 7: "ERR_CAPACITY", 8: "ERR_NO_DEVICE",
}


class Params(C.Structure):
    _fields_ = [
        ("scans_per_sweep", C.c_int32),
        ("min_tree_models", C.c_double),
        ("min_ground_models", C.c_double),
        ("max_lidar_dist", C.c_double),
        ("max_ground_lidar_dist", C.c_double),
        ("min_ground_lidar_dist", C.c_double),
        ("two_step_optim", C.c_int32),
        ("ground_radii_bins", C.c_int32),
        ("ground_theta_bins", C.c_int32),
        ("ground_retain_thresh", C.c_double),
        ("ground_match_thresh", C.c_double),
        ("rough_tree_match_thresh", C.c_double),
        ("tree_match_thresh", C.c_double),
        ("max_tree_radius", C.c_double),
        ("max_axis_theta", C.c_double),
        ("max_focus_outlier_distance", C.c_double),
        ("add_new_tree_thresh_dist", C.c_double),
        ("features_per_tree", C.c_int32),
        ("num_ground_features", C.c_int32),
        ("default_tree_radius", C.c_double),
        ("min_planes", C.c_double),
        ("beam_cluster_threshold", C.c_float),
        ("max_dist_to_centroid", C.c_float),
        ("min_vertex_size", C.c_int32),
        ("min_landmark_size", C.c_int32),
        ("min_landmark_height", C.c_float),
        ("fov_up_deg", C.c_float),
        ("fov_down_deg", C.c_float),
        ("img_w", C.c_int32),
        ("img_h", C.c_int32),
        ("do_destagger", C.c_int32),
        ("cc_dist_threshold", C.c_float),
        ("trellis_min_cluster", C.c_int32),
        ("trellis_min_beam_points", C.c_int32),
        ("trellis_min_vertices", C.c_int32),
        ("trellis_max_vertices", C.c_int32),
        ("line_ransac_thresh", C.c_double),
        ("line_ransac_max_iter", C.c_int32),
        ("line_ransac_probability", C.c_double),
        ("min_tree_height_sq", C.c_double),
        ("root_plane_max_dist", C.c_double),
        ("plane_match_thresh", C.c_double),
        ("huber_delta", C.c_double),
        ("seed", C.c_uint64),
        ("cyl_mode", C.c_int32),
        ("cyl_hypotheses", C.c_int32),
        ("cyl_inlier_thresh", C.c_float),
        ("cyl_ls_iters", C.c_int32),
        ("cyl_max_hyp_radius", C.c_float),
        ("gn_iters", C.c_int32),
        ("max_landmarks", C.c_int32),
        ("max_map", C.c_int32),
        ("max_ground", C.c_int32),
        ("batch_slots", C.c_int32),
        ("prop_samples", C.c_int32),
        ("prop_min_inlier_ratio", C.c_float),
        ("pose_solver", C.c_int32),
        ("lm_max_iters", C.c_int32),
        ("cyl_chunk_points", C.c_int32),
        ("cyl_hyp_tile", C.c_int32),
        ("cyl_queue_blocks", C.c_int32),
    ]

    def copy(self):
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def default_params(**overrides):
    """The reference's shipped configuration: params/sloam.yaml over the
    defaults of sloamNode.cpp:57-128, with the hard-coded constants of the
    path made explicit.  Mirrors sloam_params_default() in the library."""
    p = Params()
    p.scans_per_sweep = 1
    p.min_tree_models = 5
    p.min_ground_models = 36
    p.max_lidar_dist = 20.0
    p.max_ground_lidar_dist = 25.0
    p.min_ground_lidar_dist = 5.0
    p.two_step_optim = 1
    p.ground_radii_bins = 2
    p.ground_theta_bins = 18
    p.ground_retain_thresh = 0.05
    p.ground_match_thresh = 1.0
    p.rough_tree_match_thresh = 2.5
    p.tree_match_thresh = 0.5
    p.max_tree_radius = 0.3
    p.max_axis_theta = 10.0
    p.max_focus_outlier_distance = 0.5
    p.add_new_tree_thresh_dist = 1.5
    p.features_per_tree = 20
    p.num_ground_features = 5
    p.default_tree_radius = 0.2
    p.min_planes = 0.1 * 2 * 18
    p.beam_cluster_threshold = 0.5
    p.max_dist_to_centroid = 0.2
    p.min_vertex_size = 4
    p.min_landmark_size = 5
    p.min_landmark_height = 1.0
    p.fov_up_deg = 22.5
    p.fov_down_deg = -22.5
    p.img_w = 2048
    p.img_h = 64
    p.do_destagger = 1
    p.cc_dist_threshold = 1.0
    p.trellis_min_cluster = 80
    p.trellis_min_beam_points = 3
    p.trellis_min_vertices = 16
    p.trellis_max_vertices = 56
    p.line_ransac_thresh = 0.25
    p.line_ransac_max_iter = 50
    p.line_ransac_probability = 0.99
    p.min_tree_height_sq = 1.5
    p.root_plane_max_dist = 2.0
    p.plane_match_thresh = 1.0
    p.huber_delta = 0.1
    p.seed = 0
    p.cyl_mode = 0
    p.cyl_hypotheses = 256
    p.cyl_inlier_thresh = 0.03
    p.cyl_ls_iters = 3
    p.cyl_max_hyp_radius = 1.0
    p.gn_iters = 10
    p.max_landmarks = 1024
    p.max_map = 4096
    p.max_ground = 0
    p.batch_slots = 8
    p.prop_samples = 8
    p.prop_min_inlier_ratio = 0.6
    p.pose_solver = 0
    p.lm_max_iters = 50
    p.cyl_chunk_points = 256
    p.cyl_hyp_tile = 256
    p.cyl_queue_blocks = 0
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


class SE3(C.Structure):
    _fields_ = [("q", C.c_double * 4), ("t", C.c_double * 3)]

    @staticmethod
    def from_qt(q, t):
        s = SE3()
        for i in range(4):
            s.q[i] = float(q[i])
        for i in range(3):
            s.t[i] = float(t[i])
        return s

    @staticmethod
    def identity():
        return SE3.from_qt((0, 0, 0, 1), (0, 0, 0))

    def qt(self):
        return np.array(self.q[:]), np.array(self.t[:])


class Landmarks(C.Structure):
    _fields_ = [
        ("cap_landmarks", C.c_int32), ("cap_vertices", C.c_int32), ("cap_points", C.c_int32),
        ("n_landmarks", C.c_int32), ("n_vertices", C.c_int32), ("n_points", C.c_int32),
        ("tree_id", C.POINTER(C.c_int32)),
        ("vertex_begin", C.POINTER(C.c_int32)),
        ("vertex_xyz", C.POINTER(C.c_float)),
        ("vertex_radius", C.POINTER(C.c_double)),
        ("vertex_row", C.POINTER(C.c_int32)),
        ("point_begin", C.POINTER(C.c_int32)),
        ("point_xyzi", C.POINTER(C.c_float)),
        ("cap_cluster", C.c_int32), ("n_cluster", C.c_int32),
        ("cluster_begin", C.POINTER(C.c_int32)),
        ("cluster_xyzi", C.POINTER(C.c_float)),
    ]


class Cylinder(C.Structure):
    _fields_ = [("root", C.c_double * 3), ("ray", C.c_double * 3), ("radius", C.c_double),
                ("id", C.c_int32), ("valid", C.c_int32)]


class Plane(C.Structure):
    _fields_ = [("plane", C.c_double * 4), ("centroid", C.c_double * 3),
                ("bin", C.c_int32), ("valid", C.c_int32)]


class ScanOut(C.Structure):
    _fields_ = [
        ("px", C.POINTER(C.c_int32)), ("py", C.POINTER(C.c_int32)),
        ("range_image", C.POINTER(C.c_float)), ("mask_out", C.POINTER(C.c_uint8)),
        ("ground_idx", C.POINTER(C.c_int32)), ("n_ground", C.c_int32),
        ("tree_cloud", C.POINTER(C.c_float)),
    ]


class ModelsOut(C.Structure):
    _fields_ = [
        ("cap_planes", C.c_int32), ("cap_cylinders", C.c_int32),
        ("n_planes", C.c_int32), ("n_cylinders", C.c_int32),
        ("planes", C.POINTER(Plane)), ("cylinders", C.POINTER(Cylinder)),
        ("cyl_features", C.POINTER(C.c_float)), ("cyl_inliers", C.POINTER(C.c_int32)),
    ]


class RunOut(C.Structure):
    _fields_ = [
        ("models", ModelsOut), ("matches", C.POINTER(C.c_int32)),
        ("T_Map_Curr", SE3), ("T_Delta", SE3),
        ("success", C.c_int32), ("first_scan", C.c_int32),
        ("n_tree_matches", C.c_int32), ("n_plane_matches", C.c_int32),
        ("tree_check", C.c_int32), ("ground_check", C.c_int32),
    ]


# ----------------------------------------------------------------- helpers
def ptr(a, ctype):
    """Pointer to a contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


class LandmarkBuffers:
    """numpy storage behind a Landmarks struct (cap_* sized)."""

    def __init__(self, cap_lm=1024, cap_v=1024 * 56, cap_p=1 << 20, cap_cluster=0):
        self.tree_id = np.zeros(cap_lm, np.int32)
        self.vertex_begin = np.zeros(cap_lm + 1, np.int32)
        self.vertex_xyz = np.zeros(cap_v * 3, np.float32)
        self.vertex_radius = np.zeros(cap_v, np.float64)
        self.vertex_row = np.zeros(cap_v, np.int32)
        self.point_begin = np.zeros(cap_v + 1, np.int32)
        self.point_xyzi = np.zeros(cap_p * 4, np.float32)
        s = Landmarks()
        s.cap_landmarks, s.cap_vertices, s.cap_points = cap_lm, cap_v, cap_p
        s.tree_id = ptr(self.tree_id, C.c_int32)
        s.vertex_begin = ptr(self.vertex_begin, C.c_int32)
        s.vertex_xyz = ptr(self.vertex_xyz, C.c_float)
        s.vertex_radius = ptr(self.vertex_radius, C.c_double)
        s.vertex_row = ptr(self.vertex_row, C.c_int32)
        s.point_begin = ptr(self.point_begin, C.c_int32)
        s.point_xyzi = ptr(self.point_xyzi, C.c_float)
        if cap_cluster > 0:
            self.cluster_begin = np.zeros(cap_lm + 1, np.int32)
            self.cluster_xyzi = np.zeros(cap_cluster * 4, np.float32)
            s.cap_cluster = cap_cluster
            s.cluster_begin = ptr(self.cluster_begin, C.c_int32)
            s.cluster_xyzi = ptr(self.cluster_xyzi, C.c_float)
        self.s = s

    def clusters(self):
        s = self.s
        if not s.cluster_begin:
            return None
        return [self.cluster_xyzi[4 * self.cluster_begin[l]:4 * self.cluster_begin[l + 1]].reshape(-1, 4)
                for l in range(s.n_landmarks)]

    @staticmethod
    def from_trees(trees):
        """trees: list of list of dict(tree_id, xyz(3,), radius, row, points (k,4))."""
        nv = sum(len(t) for t in trees)
        npnt = sum(len(v["points"]) for t in trees for v in t)
        b = LandmarkBuffers(max(1, len(trees)), max(1, nv), max(1, npnt))
        vi = pi = 0
        for l, t in enumerate(trees):
            b.tree_id[l] = t[0]["tree_id"]
            b.vertex_begin[l] = vi
            for v in t:
                b.vertex_xyz[3 * vi:3 * vi + 3] = v["xyz"]
                b.vertex_radius[vi] = v["radius"]
                b.vertex_row[vi] = v.get("row", 0)
                b.point_begin[vi] = pi
                pts = np.asarray(v["points"], np.float32).reshape(-1, 4)
                b.point_xyzi[4 * pi:4 * (pi + len(pts))] = pts.ravel()
                pi += len(pts)
                vi += 1
        b.vertex_begin[len(trees)] = vi
        b.point_begin[vi] = pi
        b.s.n_landmarks, b.s.n_vertices, b.s.n_points = len(trees), nv, npnt
        return b

    def to_trees(self):
        s = self.s
        out = []
        for l in range(s.n_landmarks):
            t = []
            for v in range(self.vertex_begin[l], self.vertex_begin[l + 1]):
                p0, p1 = self.point_begin[v], self.point_begin[v + 1]
                t.append(dict(tree_id=int(self.tree_id[l]),
                              xyz=self.vertex_xyz[3 * v:3 * v + 3].copy(),
                              radius=float(self.vertex_radius[v]),
                              row=int(self.vertex_row[v]),
                              points=self.point_xyzi[4 * p0:4 * p1].reshape(-1, 4).copy()))
            out.append(t)
        return out


class ModelBuffers:
    def __init__(self, params, cap_planes=4096, cap_cyl=4096):
        F = params.features_per_tree
        self.planes = (Plane * cap_planes)()
        self.cylinders = (Cylinder * cap_cyl)()
        self.cyl_features = np.zeros(cap_cyl * F * 4, np.float32)
        self.cyl_inliers = np.zeros(cap_cyl, np.int32)
        self.F = F
        m = ModelsOut()
        m.cap_planes, m.cap_cylinders = cap_planes, cap_cyl
        m.planes = C.cast(self.planes, C.POINTER(Plane))
        m.cylinders = C.cast(self.cylinders, C.POINTER(Cylinder))
        m.cyl_features = ptr(self.cyl_features, C.c_float)
        m.cyl_inliers = ptr(self.cyl_inliers, C.c_int32)
        self.s = m

    def plane_array(self):
        n = self.s.n_planes
        return np.array([[*p.plane, *p.centroid, p.bin] for p in self.planes[:n]]).reshape(n, 8)

    def cyl_array(self):
        n = self.s.n_cylinders
        return np.array([[*c.root, *c.ray, c.radius, c.id] for c in self.cylinders[:n]]).reshape(n, 8)

    def features(self):
        n = self.s.n_cylinders
        return self.cyl_features[:n * self.F * 4].reshape(n, self.F, 4)


class RunBuffers:
    def __init__(self, params, cap_planes=4096, cap_cyl=4096):
        self.m = ModelBuffers(params, cap_planes, cap_cyl)
        self.matches = np.full(cap_cyl, -7, np.int32)
        r = RunOut()
        r.models = self.m.s
        r.matches = ptr(self.matches, C.c_int32)
        self.s = r

    def refresh(self):
        # copy the nested struct's counts back into the ModelBuffers view
        self.m.s.n_planes = self.s.models.n_planes
        self.m.s.n_cylinders = self.s.models.n_cylinders


def cylinders_to_array(arr, n):
    """The first n of a ctypes array of Cylinder -> (n,8) [root3, ray3, radius, id]."""
    return np.array([[*c.root, *c.ray, c.radius, c.id] for c in arr[:n]],
                    np.float64).reshape(n, 8)


def cylinders_from_array(a):
    """(n,8) [root3, ray3, radius, id] -> ctypes array of Cylinder."""
    n = len(a)
    arr = (Cylinder * max(1, n))()
    for i in range(n):
        for j in range(3):
            arr[i].root[j] = float(a[i, j])
            arr[i].ray[j] = float(a[i, 3 + j])
        arr[i].radius = float(a[i, 6])
        arr[i].id = int(a[i, 7])
        arr[i].valid = 1
    return arr
