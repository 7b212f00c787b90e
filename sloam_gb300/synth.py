"""Seeded synthetic forests and organised lidar scans.

No public dataset is named for this path, and the reference's own rosbags are
not available, so benchmark and parity inputs are synthetic: a sloped ground
plane, tilted cylindrical trunks, spherical shrubs (label 0) and outliers,
ray-cast into an organised H x W scan (row 0 = top beam, column c at azimuth
yaw_c = pi * (2 (c + 0.5) / W - 1), the inverse of the range-image
projection).  Per-point labels come from the generator (tree = 255,
ground = 1, other = 0) in place of the segmentation network.
"""
import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class SceneConfig:
    H: int = 64
    W: int = 2048
    fov_up: float = 22.5
    fov_down: float = -22.5
    n_trees_visible: int = 150       # trees inside the scan disc
    n_map: int = 400                 # landmarks in the submap (>= visible)
    disc: float = 30.0               # tree centres uniform in this disc (m)
    r_range: tuple = (0.08, 0.6)
    tilt_max_deg: float = 5.0
    h_range: tuple = (2.0, 6.0)
    slope_max_deg: float = 10.0
    sensor_height: float = 2.0
    noise: float = 0.02
    outlier_frac: float = 0.10
    background_frac: float = 0.20    # fraction of beams on shrubs (approx.)
    max_range: float = 30.0
    min_range: float = 0.1
    pose_perturb_t: float = 0.3
    pose_perturb_deg: float = 3.0


C1 = SceneConfig(H=16, W=1024, fov_up=15.0, fov_down=-15.0, n_trees_visible=20, n_map=20,
                 r_range=(0.10, 0.40), outlier_frac=0.05, background_frac=0.0)
# 64x2048 keyframe; its ground slope is drawn below the 0.1 rad plane gate of
# sloam.cpp:405-406 so that ground planes constrain the pose.
C2 = SceneConfig(slope_max_deg=4.0)


def rot_z(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])


def rot_axis(axis, ang):
    axis = np.asarray(axis, float)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * K @ K


def quat_from_R(R):
    tr = np.trace(R)
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        w, x, y, z = 0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = math.sqrt(1 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        w, x, y, z = (R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s
    elif R[1, 1] > R[2, 2]:
        s = math.sqrt(1 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        w, x, y, z = (R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s
    else:
        s = math.sqrt(1 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        w, x, y, z = (R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s
    q = np.array([x, y, z, w])
    return q / np.linalg.norm(q)


def R_from_quat(q):
    """Rotation of a quaternion (x, y, z, w); the identity for the all-zero
    pose a failed keyframe reports."""
    nq = np.linalg.norm(q)
    if not nq > 0:
        return np.eye(3)
    x, y, z, w = q / nq
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


@dataclass
class Forest:
    ground_n: np.ndarray          # unit normal of the ground plane (world)
    ground_d: float               # n.x + d = 0
    base: np.ndarray              # (T,3) trunk base on the ground
    axis: np.ndarray              # (T,3) unit axis, z > 0
    radius: np.ndarray            # (T,)
    height: np.ndarray            # (T,)
    shrub_c: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    shrub_r: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def ground_z(self, x, y):
        n, d = self.ground_n, self.ground_d
        return -(n[0] * x + n[1] * y + d) / n[2]

    def map_cylinders(self):
        """(T,8) [root3, ray3, radius, id] map models: root on the ground."""
        T = len(self.radius)
        return np.concatenate([self.base, self.axis, self.radius[:, None],
                               np.arange(T, dtype=float)[:, None]], axis=1)


def make_forest(cfg: SceneConfig, rng: np.random.Generator) -> Forest:
    slope = math.radians(rng.uniform(0, cfg.slope_max_deg))
    az = rng.uniform(0, 2 * math.pi)
    n = np.array([-math.sin(slope) * math.cos(az), -math.sin(slope) * math.sin(az), math.cos(slope)])
    d = 0.0
    # visible trees inside `disc`, the rest of the map outside it (same density)
    map_disc = cfg.disc * math.sqrt(max(cfg.n_map, cfg.n_trees_visible) / cfg.n_trees_visible)
    xs, ys = [], []
    while len(xs) < cfg.n_map:
        r = map_disc * math.sqrt(rng.uniform(0, 1))
        inside = r < cfg.disc
        n_in = sum(1 for (a, b) in zip(xs, ys) if math.hypot(a, b) < cfg.disc)
        if inside and n_in >= cfg.n_trees_visible:
            continue
        if (not inside) and (len(xs) - n_in) >= cfg.n_map - cfg.n_trees_visible:
            continue
        if r < 2.0:
            continue
        t = rng.uniform(0, 2 * math.pi)
        x, y = r * math.cos(t), r * math.sin(t)
        if any((x - a) ** 2 + (y - b) ** 2 < 1.5 ** 2 for a, b in zip(xs, ys)):
            continue
        xs.append(x)
        ys.append(y)
    T = len(xs)
    xs, ys = np.array(xs), np.array(ys)
    tilt = np.radians(rng.uniform(0, cfg.tilt_max_deg, T))
    taz = rng.uniform(0, 2 * math.pi, T)
    axis = np.stack([np.sin(tilt) * np.cos(taz), np.sin(tilt) * np.sin(taz), np.cos(tilt)], 1)
    f = Forest(n, d, None, axis, rng.uniform(*cfg.r_range, T), rng.uniform(*cfg.h_range, T))
    f.base = np.stack([xs, ys, f.ground_z(xs, ys)], 1)
    if cfg.background_frac > 0:
        ns = int(round(40 * cfg.background_frac / 0.2))
        r = cfg.disc * np.sqrt(rng.uniform(0.02, 1, ns))
        t = rng.uniform(0, 2 * math.pi, ns)
        sx, sy = r * np.cos(t), r * np.sin(t)
        sr = rng.uniform(0.4, 1.4, ns)
        f.shrub_c = np.stack([sx, sy, f.ground_z(sx, sy) + 0.5 * sr], 1)
        f.shrub_r = sr
    return f


def sensor_pose(forest: Forest, cfg: SceneConfig, rng, xy=(0.0, 0.0), yaw=None):
    """World <- sensor pose (R, t): sensor `sensor_height` above the ground."""
    if yaw is None:
        yaw = rng.uniform(-math.pi, math.pi)
    R = rot_z(yaw) @ rot_axis([1, 0, 0], math.radians(rng.normal(0, 1.0))) @ \
        rot_axis([0, 1, 0], math.radians(rng.normal(0, 1.0)))
    x, y = xy
    t = np.array([x, y, forest.ground_z(x, y) + cfg.sensor_height])
    return R, t


def perturb(R, t, cfg: SceneConfig, rng):
    dt = rng.normal(size=3)
    dt *= cfg.pose_perturb_t / np.linalg.norm(dt)
    ax = rng.normal(size=3)
    dR = rot_axis(ax, math.radians(cfg.pose_perturb_deg))
    return dR @ R, t + dt


def beam_dirs(cfg: SceneConfig):
    H, W = cfg.H, cfg.W
    fu, fd = math.radians(cfg.fov_up), math.radians(cfg.fov_down)
    pitch = fu - (np.arange(H) + 0.5) * (fu - fd) / H
    yaw = np.pi * (2 * (np.arange(W) + 0.5) / W - 1)
    az = -yaw
    cp = np.cos(pitch)[:, None]
    d = np.stack([cp * np.cos(az)[None, :], cp * np.sin(az)[None, :],
                  np.repeat(np.sin(pitch)[:, None], W, 1)], -1)
    return d.reshape(-1, 3), az


def scan(forest: Forest, R, t, cfg: SceneConfig, rng):
    """Ray-cast one organised scan.  Returns xyzi (H*W,4) float32 in the
    sensor frame (NaN where no return), labels (H*W,) uint8 and the index of
    the tree hit per beam (-1 none)."""
    H, W = cfg.H, cfg.W
    D, az = beam_dirs(cfg)          # sensor frame
    N = H * W
    best = np.full(N, np.inf)
    label = np.zeros(N, np.uint8)
    tree_hit = np.full(N, -1, np.int32)
    Rt = R.T
    # ground
    n_s = Rt @ forest.ground_n
    d_s = forest.ground_d + forest.ground_n @ t
    den = D @ n_s
    with np.errstate(divide="ignore", invalid="ignore"):
        tg = -d_s / den
    ok = (den < 0) & (tg > 0)
    best[ok] = tg[ok]
    label[ok] = 1
    # trunks, each tested only on its azimuth window
    base_s = (forest.base - t) @ R         # rows: R^T (p - t)
    axis_s = forest.axis @ R
    for k in range(len(forest.radius)):
        b, a, r, h = base_s[k], axis_s[k], forest.radius[k], forest.height[k]
        dist = math.hypot(b[0], b[1])
        if dist > cfg.max_range + r or dist < r + 0.2:
            continue
        c_az = math.atan2(b[1], b[0])
        half = math.asin(min(1.0, (r + 0.05) / dist)) + 1e-3
        cols = _cols_in(az, c_az, half)
        if cols.size == 0:
            continue
        idx = (np.arange(H)[:, None] * W + cols[None, :]).ravel()
        Dk = D[idx]
        dp = Dk - (Dk @ a)[:, None] * a
        w = -b
        wp = w - (w @ a) * a
        A_ = np.einsum("ij,ij->i", dp, dp)
        B_ = dp @ wp
        C_ = wp @ wp - r * r
        disc = B_ * B_ - A_ * C_
        good = disc >= 0
        with np.errstate(invalid="ignore", divide="ignore"):
            tt = (-B_ - np.sqrt(np.where(good, disc, 0))) / A_
        s = (tt[:, None] * Dk - b) @ a
        hit = good & (tt > 0) & (s >= 0) & (s <= h) & (tt < best[idx])
        sel = idx[hit]
        best[sel] = tt[hit]
        label[sel] = 255
        tree_hit[sel] = k
    # shrubs (label 0)
    if len(forest.shrub_r):
        cs = (forest.shrub_c - t) @ R
        for k in range(len(forest.shrub_r)):
            c, r = cs[k], forest.shrub_r[k]
            dist = np.linalg.norm(c)
            if dist > cfg.max_range + r or dist < r + 0.2:
                continue
            c_az = math.atan2(c[1], c[0])
            half = math.asin(min(1.0, r / math.hypot(c[0], c[1]) if math.hypot(c[0], c[1]) > r else 1.0)) + 1e-3
            cols = _cols_in(az, c_az, half)
            idx = (np.arange(H)[:, None] * W + cols[None, :]).ravel()
            Dk = D[idx]
            bb = Dk @ c
            cc = c @ c - r * r
            disc = bb * bb - cc
            good = disc >= 0
            tt = bb - np.sqrt(np.where(good, disc, 0))
            hit = good & (tt > 0) & (tt < best[idx])
            sel = idx[hit]
            best[sel] = tt[hit]
            label[sel] = 0
            tree_hit[sel] = -1
    valid = np.isfinite(best) & (best <= cfg.max_range) & (best >= cfg.min_range)
    rng_noise = rng.normal(0, cfg.noise, N)
    rr = best + rng_noise
    # outliers: trunk beams move up to +-1 m along the beam (stay labelled
    # tree: segmentation noise inside the cluster); other beams return early
    # (dust, vegetation in front: uniform range before the surface) and keep
    # their label
    out = valid & (rng.uniform(0, 1, N) < cfg.outlier_frac)
    on_tree = out & (label == 255)
    rr[on_tree] = best[on_tree] + rng.uniform(-1.0, 1.0, on_tree.sum())
    other = out & (label != 255)
    rr[other] = rng.uniform(cfg.min_range, 1.0, other.sum()) * best[other]
    xyz = D * rr[:, None]
    xyzi = np.empty((N, 4), np.float32)
    xyzi[:, :3] = xyz
    xyzi[:, 3] = rng.uniform(0, 255, N).astype(np.float32)
    xyzi[~valid, :3] = np.nan
    label[~valid] = 0
    tree_hit[~valid] = -1
    return xyzi, label, tree_hit


def _cols_in(az, c_az, half):
    dd = np.angle(np.exp(1j * (az - c_az)))
    return np.nonzero(np.abs(dd) <= half)[0]


@dataclass
class Keyframe:
    xyzi: np.ndarray
    labels: np.ndarray
    tree_hit: np.ndarray
    R_gt: np.ndarray
    t_gt: np.ndarray
    R_est: np.ndarray
    t_est: np.ndarray

    def pose_est_qt(self):
        return quat_from_R(self.R_est), self.t_est

    def pose_gt_qt(self):
        return quat_from_R(self.R_gt), self.t_gt


def make_keyframe(forest: Forest, cfg: SceneConfig, rng, xy=(0.0, 0.0), yaw=None) -> Keyframe:
    R, t = sensor_pose(forest, cfg, rng, xy, yaw)
    xyzi, lab, th = scan(forest, R, t, cfg, rng)
    Re, te = perturb(R, t, cfg, rng)
    return Keyframe(xyzi, lab, th, R, t, Re, te)


def scene(cfg: SceneConfig = C2, seed: int = 0, n_kf: int = 1):
    """A forest and n_kf keyframes taken at random yaw from the origin."""
    rng = np.random.default_rng(seed)
    forest = make_forest(cfg, rng)
    kfs = [make_keyframe(forest, cfg, rng) for _ in range(n_kf)]
    return forest, kfs


def preset_params(cfg: SceneConfig, base=None, **kw):
    """Reference parameters adjusted so the reference algorithm can accept the
    synthetic scenes: max_tree_radius above the largest trunk, max_lidar_dist
    beyond the scan disc, the Trellis minimum vertex count below H, no Ouster
    destagger (the synthetic sensor is not staggered), and at least 16 plane
    feature matches (more than 3 matched planes) for the pose instead of 37.
    The keyframes of a synthetic scene stand at scattered places of the
    forest, so only a few of a keyframe's ground bins lie within the 1 m
    plane-match distance of the first scan's (sloam.cpp:490), and the plane
    gate drops every bin whose SVD normal comes out pointing down
    (sloam.cpp:402-406): about 6 planes of a 64x2048 keyframe match."""
    from .capi import default_params
    p = default_params() if base is None else base.copy()
    p.img_h, p.img_w = cfg.H, cfg.W
    p.fov_up_deg, p.fov_down_deg = cfg.fov_up, cfg.fov_down
    p.do_destagger = 0
    p.max_tree_radius = max(0.3, cfg.r_range[1] + 0.2)
    p.max_lidar_dist = cfg.disc + 5.0
    p.trellis_min_vertices = min(16, max(3, cfg.H // 2 - 1))
    p.min_ground_models = min(p.min_ground_models, 15.0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


# ------------------------------------------------------------ uneven batch
# 64 keyframes of 64x2048, tree counts log-uniform in 20-400 per keyframe,
# cluster sizes from tens of points (far, thin trunks) to ~20k (a thick trunk
# a metre from the sensor).  Each keyframe sits at the centre of its own
# 80 m cell of one forest (cells are beyond each other's 30 m range); the map
# holds every tree of every cell.
C3 = SceneConfig(slope_max_deg=2.0, disc=28.0)
C3_CELL = 80.0


def c3_scene(seed: int = 0, n_kf: int = 64, counts=None):
    """(forest, keyframes, tree counts).  `counts` overrides the drawn tree
    count of each keyframe."""
    cfg = C3
    rng = np.random.default_rng(seed)
    if counts is None:
        counts = np.round(np.exp(rng.uniform(math.log(20), math.log(400), n_kf))).astype(int)
    counts = [int(c) for c in counts]
    slope = math.radians(rng.uniform(0, cfg.slope_max_deg))
    az = rng.uniform(0, 2 * math.pi)
    n = np.array([-math.sin(slope) * math.cos(az), -math.sin(slope) * math.sin(az),
                  math.cos(slope)])
    side = int(math.ceil(math.sqrt(len(counts))))
    centres = [(C3_CELL * (k % side), C3_CELL * (k // side)) for k in range(len(counts))]
    xs, ys = [], []
    for (cx, cy), T in zip(centres, counts):
        cell = []
        # one trunk close to the sensor per cell (the large clusters)
        while len(cell) < T:
            r = (1.2 + 0.8 * rng.uniform()) if not cell else cfg.disc * math.sqrt(rng.uniform(0.004, 1))
            t = rng.uniform(0, 2 * math.pi)
            x, y = r * math.cos(t), r * math.sin(t)
            if any((x - a) ** 2 + (y - b) ** 2 < 1.5 ** 2 for a, b in cell):
                continue
            cell.append((x, y))
        xs += [cx + a for a, _ in cell]
        ys += [cy + b for _, b in cell]
    T = len(xs)
    xs, ys = np.array(xs), np.array(ys)
    tilt = np.radians(rng.uniform(0, cfg.tilt_max_deg, T))
    taz = rng.uniform(0, 2 * math.pi, T)
    axis = np.stack([np.sin(tilt) * np.cos(taz), np.sin(tilt) * np.sin(taz), np.cos(tilt)], 1)
    f = Forest(n, 0.0, None, axis, rng.uniform(*cfg.r_range, T), rng.uniform(*cfg.h_range, T))
    f.base = np.stack([xs, ys, f.ground_z(xs, ys)], 1)
    near = np.cumsum([0] + counts[:-1])  # the first trunk of each cell
    f.radius[near] = rng.uniform(0.45, 0.6, len(near))
    f.height[near] = rng.uniform(5.0, 6.0, len(near))
    sc, sr = [], []
    for cx, cy in centres:
        r = cfg.disc * np.sqrt(rng.uniform(0.02, 1, 40))
        t = rng.uniform(0, 2 * math.pi, 40)
        sx, sy = cx + r * np.cos(t), cy + r * np.sin(t)
        rr = rng.uniform(0.4, 1.4, 40)
        sc.append(np.stack([sx, sy, f.ground_z(sx, sy) + 0.5 * rr], 1))
        sr.append(rr)
    f.shrub_c, f.shrub_r = np.concatenate(sc), np.concatenate(sr)
    kfs = [make_keyframe(f, cfg, rng, xy=c) for c in centres]
    return f, kfs, counts


def c3_params(forest: Forest, base=None, **kw):
    """C2's reference presets with capacities for the uneven batch: every
    tree of the forest in the map, up to 400 trees (plus shrub blobs) per
    keyframe."""
    p = preset_params(C3, base, **kw)
    p.max_map = max(p.max_map, len(forest.radius))
    p.max_landmarks = max(p.max_landmarks, 1024)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def cylinder_errors(forest: Forest, cyl, max_dist=0.5):
    """Fitted cylinders (rows [root3, ray3, radius, id], map frame) against
    the forest's trunks.  Each is matched to the trunk whose axis passes
    nearest its root (horizontal distance at the root's height, at most
    max_dist).  Returns (axis angle in degrees, |radius error| in m) per
    matched cylinder."""
    angs, rerrs = [], []
    base, axis, rad = forest.base, forest.axis, forest.radius
    for c in np.asarray(cyl, float).reshape(-1, 8):
        root, ray = c[:3], c[3:6] / np.linalg.norm(c[3:6])
        t = (root[2] - base[:, 2]) / axis[:, 2]
        p = base + t[:, None] * axis
        d = np.hypot(p[:, 0] - root[0], p[:, 1] - root[1])
        k = int(np.argmin(d))
        if d[k] > max_dist:
            continue
        angs.append(math.degrees(math.acos(min(1.0, abs(float(ray @ axis[k]))))))
        rerrs.append(abs(c[6] - rad[k]))
    return np.array(angs), np.array(rerrs)
