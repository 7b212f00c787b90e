"""The long-trajectory scenes and the reference's map-manager loop: path,
terrain and forest properties, the map manager's submap and update rules
(mapManager.cpp:8-70), and a short sequence through the GPU path and the
oracle."""
import math

import numpy as np
import pytest

from sloam_gb300 import trajectory as TJ


def test_path_steps_and_yaw_rate():
    rng = np.random.default_rng(0)
    p = TJ.make_path(200, rng)
    steps = np.linalg.norm(np.diff(p[:, :2], axis=0), axis=1)
    assert np.allclose(steps, 1.0)
    dyaw = np.degrees(np.abs(np.angle(np.exp(1j * np.diff(p[1:, 2])))))
    assert dyaw.max() <= 15.0 + 1e-9


def test_terrain_is_planar_facets_within_slope():
    rng = np.random.default_rng(1)
    path = TJ.make_path(200, rng)
    ter = TJ.make_terrain(path, rng)
    # every facet's gradient is at most tan(20 deg)
    h, c = ter.h, ter.cell
    gx = np.abs(np.diff(h, axis=0)) / c
    gy = np.abs(np.diff(h, axis=1)) / c
    assert max(gx.max(), gy.max()) <= math.tan(math.radians(20)) + 1e-9
    # linear inside a facet: the midpoint of two points of one triangle
    x0, y0 = ter.x0 + 3.0, ter.y0 + 4.0
    x1, y1 = ter.x0 + 5.0, ter.y0 + 2.0
    za, zb = ter.z(np.array([x0, x1]), np.array([y0, y1]))
    zm = ter.z(np.array([(x0 + x1) / 2]), np.array([(y0 + y1) / 2]))[0]
    assert abs(zm - (za + zb) / 2) < 1e-9


def test_forest_corridor():
    rng = np.random.default_rng(2)
    path = TJ.make_path(50, rng)
    ter = TJ.make_terrain(path, rng)
    f = TJ.make_forest(path, ter, rng, n_trees=150)
    d = np.min(np.hypot(f.base[:, None, 0] - path[None, :, 0], f.base[:, None, 1] - path[None, :, 1]), 1)
    assert len(f.radius) == 150 and d.max() <= 35.0 and d.min() >= 2.5
    assert np.allclose(f.base[:, 2], ter.z(f.base[:, 0], f.base[:, 1]))


def test_map_manager_rules():
    mm = TJ.MapManager(k=3, recent=5)
    assert len(mm.submap([0, 0, 0])) == 0
    cyl = np.array([[x, 0.0, 0.0, 0, 0, 1, 0.2, i] for i, x in enumerate([5.0, 1.0, 3.0, 9.0, 7.0])])
    mm.update(cyl, [-1] * 5)
    assert mm.hits == [1] * 5
    sub = mm.submap([0.0, 0.0, 0.0])
    # the 3 nearest (1, 3, 5 m), but index 0 (5 m) is not among the 5 - 1 most
    # recent (map_size - index < recent)
    assert [int(c[7]) for c in sub] == [1, 2]
    assert mm.matches_map == {0: 1, 1: 2}
    upd = sub[1].copy()
    upd[0] = 3.5
    mm.update(np.array([upd]), [1])
    assert mm.hits[2] == 2 and mm.roots[2, 0] == 3.5 and mm.matches_map == {}


def test_scene_scan_on_cpu():
    poses, odo, forest, ter, scans = TJ.scene(seed=3, n_kf=2, H=16, W=256, n_trees=120)
    xyzi, lab = scans[0]
    assert xyzi.shape == (16 * 256, 4) and lab.shape == (16 * 256,)
    assert (lab == 1).any() and (lab == 255).any()
    assert len(odo) == 1


@pytest.mark.gpu
def test_short_trajectory_gpu_and_oracle():
    import ctypes as C
    from oracle import loader
    import trajectory_run
    from sloam_gb300.lib import Context
    poses, odo, forest, ter, scans = TJ.scene(seed=0, n_kf=12, H=64, W=1024, n_trees=300,
                                              device="cuda")
    P = TJ.params(64, 1024, 1, submap=300)
    ctx = Context(P)
    est_g, _ = TJ.run(TJ.gpu_keyframe_fn(ctx), P, poses, odo, scans, 300)
    ctx.close()
    L = loader.lib()
    s = L.oracle_create(C.byref(P))
    est_o, _ = TJ.run(trajectory_run.oracle_keyframe_fn(L, s), P, poses, odo, scans, 300)
    L.oracle_destroy(s)
    dg, do = TJ.drift(poses, est_g), TJ.drift(poses, est_o)
    print(dg, do)
    # the same algorithm: the two trajectories agree closely
    te_g = np.array([e[1] for e in est_g])
    te_o = np.array([e[1] for e in est_o])
    assert np.abs(te_g - te_o).max() < 1e-3
    assert dg["ate_rmse_m"] < 0.5
