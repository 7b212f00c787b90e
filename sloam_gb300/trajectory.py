"""Long-trajectory evaluation: sequential keyframes along a smooth path
through a forest on piecewise-planar terrain, each keyframe run the way
SLOAMNode::run does it (sloamNode.cpp:186-282): pose estimate = previous
estimated pose composed with an odometry increment, submap query, keyframe,
map update.  The scene generator, the host map manager, the keyframe loop
and the drift figures live here; `trajectory_run.py` (beside `bench.py`)
runs them on the GPU path and on the CPU restatement of the reference.

Scenes (configuration 5 of the benchmark set): 200 keyframes of 128x2048,
1 m per keyframe, yaw rate at most 15 deg per keyframe, a 1 000-tree forest
on a triangulated height field (planar facets, slope at most 20 deg), a
1 000-landmark submap, 15 Gauss-Newton iterations.  The scans are ray-cast
with PyTorch on the device given (the GPU for full size), a data generator
only.
"""
import ctypes as C
import math
import time

import numpy as np

from . import synth


# ------------------------------------------------------------------ scene
class Terrain:
    """Height field on a grid of `cell` metres; each cell is two planar
    triangles (split along u + v = 1)."""

    def __init__(self, x0, y0, nx, ny, cell, heights):
        self.x0, self.y0, self.nx, self.ny, self.cell = x0, y0, nx, ny, cell
        self.h = heights  # (nx + 1, ny + 1)

    def z(self, x, y, xp=np):
        u = (x - self.x0) / self.cell
        v = (y - self.y0) / self.cell
        i = xp.clip(xp.floor(u), 0, self.nx - 1)
        j = xp.clip(xp.floor(v), 0, self.ny - 1)
        fu, fv = u - i, v - j
        h = self.h if xp is np else self._th
        ii, jj = (i.astype(int), j.astype(int)) if xp is np else (i.long(), j.long())
        h00, h10, h01, h11 = h[ii, jj], h[ii + 1, jj], h[ii, jj + 1], h[ii + 1, jj + 1]
        low = fu + fv < 1
        za = h00 + fu * (h10 - h00) + fv * (h01 - h00)
        zb = h11 + (1 - fu) * (h01 - h11) + (1 - fv) * (h10 - h11)
        return xp.where(low, za, zb)

    def to(self, torch, device):
        self._th = torch.as_tensor(self.h, dtype=torch.float64, device=device)
        return self


def make_path(n, rng, step=1.0, max_yaw_deg=15.0):
    """n poses (x, y, yaw): 1 m steps, a yaw rate that wanders smoothly and
    stays within +-max_yaw_deg per keyframe."""
    w, th = 0.0, rng.uniform(-math.pi, math.pi)
    p = np.zeros((n, 3))
    for k in range(1, n):
        w = float(np.clip(w + math.radians(rng.uniform(-4, 4)), -math.radians(max_yaw_deg),
                          math.radians(max_yaw_deg)))
        th += w
        p[k] = p[k - 1] + [step * math.cos(th), step * math.sin(th), 0.0]
        p[k, 2] = th
    p[0, 2] = p[1, 2] if n > 1 else th
    return p


def make_terrain(path, rng, cell=25.0, margin=45.0, max_slope_deg=20.0):
    x0, y0 = path[:, 0].min() - margin, path[:, 1].min() - margin
    nx = int(math.ceil((path[:, 0].max() + margin - x0) / cell))
    ny = int(math.ceil((path[:, 1].max() + margin - y0) / cell))
    # smooth random heights: a few random planes summed, then the slope of
    # every facet limited by scaling
    gx, gy = np.meshgrid(np.arange(nx + 1) * cell, np.arange(ny + 1) * cell, indexing="ij")
    h = np.zeros_like(gx)
    for _ in range(4):
        k = rng.uniform(0.01, 0.04, 2)
        h += rng.uniform(3, 9) * np.sin(k[0] * gx + rng.uniform(0, 6)) * np.cos(k[1] * gy + rng.uniform(0, 6))
    slope = max(np.abs(np.diff(h, axis=0)).max(), np.abs(np.diff(h, axis=1)).max(),
                np.abs(h[1:, 1:] - h[:-1, :-1]).max() / math.sqrt(2)) / cell
    lim = math.tan(math.radians(max_slope_deg)) * 0.95
    if slope > lim:
        h *= lim / slope
    return Terrain(x0, y0, nx, ny, cell, h)


def make_forest(path, terrain, rng, n_trees=1000, corridor=35.0, cfg=synth.C2):
    xs, ys = [], []
    lo, hi = path[:, :2].min(0) - corridor, path[:, :2].max(0) + corridor
    pts = path[:, :2]
    while len(xs) < n_trees:
        q = rng.uniform(lo, hi)
        d = np.hypot(*(pts - q).T).min()
        if d > corridor or d < 2.5:
            continue
        if xs and np.hypot(np.array(xs) - q[0], np.array(ys) - q[1]).min() < 1.5:
            continue
        xs.append(q[0])
        ys.append(q[1])
    T = len(xs)
    xs, ys = np.array(xs), np.array(ys)
    tilt = np.radians(rng.uniform(0, cfg.tilt_max_deg, T))
    taz = rng.uniform(0, 2 * math.pi, T)
    axis = np.stack([np.sin(tilt) * np.cos(taz), np.sin(tilt) * np.sin(taz), np.cos(tilt)], 1)
    base = np.stack([xs, ys, terrain.z(xs, ys)], 1)
    f = synth.Forest(np.array([0, 0, 1.0]), 0.0, base, axis, rng.uniform(*cfg.r_range, T),
                     rng.uniform(4.0, 8.0, T))
    return f


def ray_cast(torch, device, terrain, forest, R, t, H, W, fov_up, fov_down, rng_seed,
             noise=0.02, outlier_frac=0.10, max_range=30.0, min_range=0.1):
    """One organised H x W scan (sensor frame): trunks and the terrain;
    returns xyzi float32 (N,4) and labels uint8 (N,) as numpy."""
    fu, fd = math.radians(fov_up), math.radians(fov_down)
    pitch = fu - (torch.arange(H, device=device, dtype=torch.float64) + 0.5) * (fu - fd) / H
    yaw = math.pi * (2 * (torch.arange(W, device=device, dtype=torch.float64) + 0.5) / W - 1)
    az = -yaw
    cp = torch.cos(pitch)[:, None]
    D = torch.stack([cp * torch.cos(az)[None], cp * torch.sin(az)[None],
                     torch.sin(pitch)[:, None].expand(H, W)], -1).reshape(-1, 3)
    N = H * W
    Rt = torch.as_tensor(R, dtype=torch.float64, device=device)
    tt = torch.as_tensor(t, dtype=torch.float64, device=device)
    Dw = D @ Rt.T                                   # world directions
    best = torch.full((N,), float("inf"), dtype=torch.float64, device=device)
    label = torch.zeros(N, dtype=torch.uint8, device=device)
    # terrain: march 0.25 m steps, refine linearly at the first crossing
    steps = torch.arange(1, int(max_range / 0.25) + 1, device=device, dtype=torch.float64) * 0.25
    prev_d = None
    hit_t = torch.full((N,), float("inf"), dtype=torch.float64, device=device)
    for k in range(len(steps)):
        s = steps[k]
        p = tt + s * Dw
        d = p[:, 2] - terrain.z(p[:, 0], p[:, 1], xp=torch)
        if prev_d is not None:
            cross = (prev_d > 0) & (d <= 0) & torch.isinf(hit_t)
            if cross.any():
                s0 = s - 0.25
                frac = prev_d[cross] / (prev_d[cross] - d[cross])
                hit_t[cross] = s0 + 0.25 * frac
        prev_d = d
    g = torch.isfinite(hit_t)
    best[g] = hit_t[g]
    label[g] = 1
    # trunks within range of the sensor
    b = forest.base - t
    near = np.nonzero(np.hypot(b[:, 0], b[:, 1]) < max_range + 1.0)[0]
    if len(near):
        base = torch.as_tensor(forest.base[near], dtype=torch.float64, device=device)
        ax = torch.as_tensor(forest.axis[near], dtype=torch.float64, device=device)
        rad = torch.as_tensor(forest.radius[near], dtype=torch.float64, device=device)
        hgt = torch.as_tensor(forest.height[near], dtype=torch.float64, device=device)
        for c0 in range(0, len(near), 64):
            sl = slice(c0, c0 + 64)
            a = ax[sl]                                  # (T,3)
            w0 = tt - base[sl]                          # (T,3) from base to sensor
            dp = Dw[:, None, :] - (Dw @ a.T)[:, :, None] * a[None]   # (N,T,3)
            wp = w0 - (w0 * a).sum(1, keepdim=True) * a              # (T,3)
            A_ = (dp * dp).sum(-1)
            B_ = (dp * wp[None]).sum(-1)
            C_ = (wp * wp).sum(-1)[None] - rad[sl][None] ** 2
            disc = B_ * B_ - A_ * C_
            ok = disc >= 0
            tq = (-B_ - torch.sqrt(torch.clamp(disc, min=0))) / A_
            sa = ((tq[..., None] * Dw[:, None, :] + w0[None]) * a[None]).sum(-1)
            hit = ok & (tq > 0) & (sa >= 0) & (sa <= hgt[sl][None])
            tq = torch.where(hit, tq, torch.full_like(tq, float("inf")))
            tmin, _ = tq.min(1)
            closer = tmin < best
            best[closer] = tmin[closer]
            label[closer] = 255
    gen = torch.Generator(device=device)
    gen.manual_seed(int(rng_seed))
    valid = torch.isfinite(best) & (best <= max_range) & (best >= min_range)
    rr = best + noise * torch.randn(N, generator=gen, device=device, dtype=torch.float64)
    out = valid & (torch.rand(N, generator=gen, device=device, dtype=torch.float64) < outlier_frac)
    on_tree = out & (label == 255)
    rr[on_tree] = best[on_tree] + (2 * torch.rand(int(on_tree.sum()), generator=gen, device=device,
                                                  dtype=torch.float64) - 1)
    other = out & (label != 255)
    rr[other] = (min_range + (1 - min_range) * torch.rand(int(other.sum()), generator=gen,
                                                          device=device, dtype=torch.float64)) * best[other]
    xyz = D * rr[:, None]
    xyzi = torch.empty((N, 4), dtype=torch.float32, device=device)
    xyzi[:, :3] = xyz.float()
    xyzi[:, 3] = 100.0
    xyzi[~valid, :3] = float("nan")
    label[~valid] = 0
    return xyzi.cpu().numpy(), label.cpu().numpy()


def scene(seed=0, n_kf=200, H=128, W=2048, n_trees=1000, device="cpu"):
    """(path poses (R, t) per keyframe, odometry increments, forest, terrain,
    scans) of the long trajectory."""
    import torch
    rng = np.random.default_rng(seed)
    path = make_path(n_kf, rng)
    terrain = make_terrain(path, rng)
    forest = make_forest(path, terrain, rng, n_trees)
    terrain.to(torch, device)
    poses = []
    for k in range(n_kf):
        x, y, th = path[k]
        R = synth.rot_z(th) @ synth.rot_axis([1, 0, 0], math.radians(rng.normal(0, 1.0))) @ \
            synth.rot_axis([0, 1, 0], math.radians(rng.normal(0, 1.0)))
        t = np.array([x, y, float(terrain.z(np.array([x]), np.array([y]))[0]) + 2.0])
        poses.append((R, t))
    # odometry: the true increment with noise (0.05 m, 0.5 deg per keyframe)
    odo = []
    for k in range(1, n_kf):
        (R0, t0), (R1, t1) = poses[k - 1], poses[k]
        dR = R0.T @ R1
        dt = R0.T @ (t1 - t0)
        dR = dR @ synth.rot_axis(rng.normal(size=3), math.radians(0.5))
        dt = dt + rng.normal(0, 0.05, 3)
        odo.append((dR, dt))
    scans = [ray_cast(torch, device, terrain, forest, R, t, H, W, 22.5, -22.5, seed * 100003 + k)
             for k, (R, t) in enumerate(poses)]
    return poses, odo, forest, terrain, scans


# ---------------------------------------------------------- map manager
class MapManager:
    """The reference's map manager (mapManager.cpp:8-70): tree roots and
    models, hit counts; the submap is the k nearest roots to (x, y, 1) of
    the pose among the 200 most recently added (k = 100 in the reference;
    the benchmark's long trajectory uses a 1 000-landmark submap)."""

    def __init__(self, k=100, recent=200):
        self.k, self.recent = k, recent
        self.roots = np.zeros((0, 3))
        self.models = np.zeros((0, 8))
        self.hits = []
        self.matches_map = {}

    def submap(self, t):
        self.matches_map = {}
        if not len(self.roots):
            return np.zeros((0, 8))
        d = ((self.roots - [t[0], t[1], 1.0]) ** 2).sum(1).astype(np.float32)
        order = np.lexsort((np.arange(len(d)), d))[:self.k]
        out, n = [], len(self.models)
        for idx in order:
            if n - idx < self.recent:
                self.matches_map[len(out)] = int(idx)
                out.append(self.models[idx])
        return np.array(out).reshape(-1, 8)

    def update(self, cyl, matches):
        for c, m in zip(cyl, matches):
            if m == -1:
                self.roots = np.vstack([self.roots, c[:3]])
                self.models = np.vstack([self.models, c])
                self.hits.append(1)
            else:
                idx = self.matches_map.get(int(m), 0)
                self.roots[idx] = c[:3]
                self.models[idx] = c
                self.hits[idx] += 1
        self.matches_map = {}


def _compose(Ra, ta, Rb, tb):
    return Ra @ Rb, Ra @ tb + ta


def run(keyframe, P, poses, odo, scans, submap_k, mm=None):
    """Runs the sequence through keyframe(P, xyzi, labels, (R, t), map) ->
    (status, success, (R, t), cylinders, matches); returns the estimated
    trajectory and the wall time.  `mm`: the host map manager to use (a new
    one with k = submap_k by default)."""
    from . import capi as A
    if mm is None:
        mm = MapManager(k=submap_k)
    est = [poses[0]]
    t0 = time.perf_counter()
    for k in range(len(poses)):
        if k == 0:
            guess = poses[0]
        else:
            guess = _compose(est[-1][0], est[-1][1], *odo[k - 1])
        mp = mm.submap(guess[1])
        xyzi, lab = scans[k]
        st, ok, pose, cyl, matches = keyframe(P, xyzi, lab, guess, mp)
        if st in (0, A.SLOAM_ERR_NOT_CONVERGED):
            mm.update(cyl, matches)
        if k > 0:
            est.append(pose if (st == 0 and ok) else guess)
    return est, time.perf_counter() - t0


def run_mapped(ctx, mm, P, poses, odo, scans):
    """The same sequence through sloam_keyframe_mapped: the map manager on
    the GPU (getSubmap, RunSloam, updateMap without the map leaving the
    device).  Returns the estimated trajectory and the wall time."""
    from . import capi as A
    est = [poses[0]]
    t0 = time.perf_counter()
    for k in range(len(poses)):
        if k == 0:
            guess = poses[0]
        else:
            guess = _compose(est[-1][0], est[-1][1], *odo[k - 1])
        xyzi, lab = scans[k]
        r = A.RunBuffers(P)
        st = ctx.L.sloam_keyframe_mapped(
            ctx.h, mm.h, A.ptr(xyzi, C.c_float), len(xyzi), A.ptr(lab, C.c_uint8), None,
            C.byref(A.SE3.from_qt(synth.quat_from_R(guess[0]), guess[1])), C.byref(r.s))
        r.refresh()
        q, t = r.s.T_Map_Curr.qt()
        if k > 0:
            est.append((synth.R_from_quat(q), t) if (st == 0 and r.s.success) else guess)
    return est, time.perf_counter() - t0


def drift(poses, est):
    tr = np.array([p[1] for p in poses])
    te = np.array([e[1] for e in est])
    err = np.linalg.norm(tr - te, axis=1)
    length = float(np.linalg.norm(np.diff(tr[:, :2], axis=0), axis=1).sum())
    Rf = poses[-1][0].T @ est[-1][0]
    rot = math.degrees(math.acos(min(1.0, max(-1.0, (np.trace(Rf) - 1) / 2))))
    return {"final_translation_error_m": float(err[-1]), "path_length_m": length,
            "drift_pct": 100.0 * float(err[-1]) / max(length, 1e-9),
            "ate_rmse_m": float(np.sqrt((err ** 2).mean())), "max_error_m": float(err.max()),
            "final_rotation_error_deg": rot}


def gpu_keyframe_fn(ctx):
    from . import capi as A

    def kf(P, xyzi, lab, pose, mp):
        r = A.RunBuffers(P)
        mapc = A.cylinders_from_array(mp) if len(mp) else None
        st = ctx.L.sloam_keyframe(ctx.h, A.ptr(xyzi, C.c_float), len(xyzi), A.ptr(lab, C.c_uint8),
                                  None, C.byref(A.SE3.from_qt(synth.quat_from_R(pose[0]), pose[1])),
                                  mapc, len(mp), C.byref(r.s))
        r.refresh()
        q, t = r.s.T_Map_Curr.qt()
        n = r.s.models.n_cylinders
        return st, r.s.success, (synth.R_from_quat(q), t), r.m.cyl_array()[:n], r.matches[:n]
    return kf


def params(H, W, cyl_mode, gn_iters=15, submap=1000):
    cfg = synth.SceneConfig(H=H, W=W, disc=30.0)
    # the reference's default two-step pose (sloam.yaml): on slopes above the
    # 0.1 rad plane gate the trees alone still fix x, y and yaw
    return synth.preset_params(cfg, two_step_optim=1, cyl_mode=cyl_mode, gn_iters=gn_iters,
                               max_map=max(submap, 128), batch_slots=1)
