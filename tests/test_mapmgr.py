"""The map manager on the GPU (csrc/mapmgr.cu; MapManager,
mapManager.cpp:8-70) against the host restatement of the same rules
(sloam_gb300.trajectory.MapManager): the submap (k nearest of the map by
float distance to (x, y, 1), ties to the lower index, then only the `recent`
newest) and, through a short keyframe sequence, the update (appends,
overwrites, hit counts) and the poses."""
import numpy as np
import pytest

from sloam_gb300 import trajectory as TJ

pytestmark = pytest.mark.gpu


def _random_map(rng, n):
    roots = np.c_[rng.uniform(-40, 40, (n, 2)), rng.uniform(-1, 3, n)]
    # exact ties: repeated roots, and roots mirrored about the query point
    roots[5:40:5] = roots[4]
    rays = np.c_[rng.normal(0, 0.05, (n, 2)), np.ones(n)]
    rays /= np.linalg.norm(rays, axis=1, keepdims=True)
    models = np.c_[roots, rays, rng.uniform(0.1, 0.5, n), np.arange(n)]
    hits = rng.integers(1, 5, n).astype(np.int32)
    return models, hits


def _host(models, hits, k, recent):
    mm = TJ.MapManager(k=k, recent=recent)
    mm.roots = models[:, :3].copy()
    mm.models = models.copy()
    mm.hits = list(int(h) for h in hits)
    return mm


@pytest.mark.parametrize("n,k,recent", [(0, 100, 200), (37, 100, 200), (700, 100, 200),
                                        (700, 1000, 200), (300, 20, 50)])
def test_submap_matches_host_rules(n, k, recent):
    from sloam_gb300.lib import DeviceMapManager
    rng = np.random.default_rng(n + k)
    models, hits = _random_map(rng, n) if n else (np.zeros((0, 8)), np.zeros(0, np.int32))
    dm = DeviceMapManager(capacity=max(n, 1), k=k, recent=recent)
    dm.load(models, hits)
    for (x, y) in [(0.0, 0.0), (12.5, -3.0), (float(models[4, 0]) if n else 1.0, 2.0)]:
        host = _host(models, hits, k, recent)
        want = host.submap([x, y, 0.0])
        got, idx = dm.submap(x, y)
        assert got.shape == want.shape
        assert np.array_equal(got, want)
        assert list(idx) == [host.matches_map[i] for i in range(len(idx))]
    m2, h2 = dm.read()
    assert np.array_equal(m2, models) and np.array_equal(h2, hits)
    dm.close()


def test_mapped_sequence_matches_host_map_manager():
    from sloam_gb300.lib import Context, DeviceMapManager
    poses, odo, forest, ter, scans = TJ.scene(seed=0, n_kf=10, H=64, W=1024, n_trees=300,
                                              device="cuda")
    P = TJ.params(64, 1024, 1, submap=300)
    host_mm = TJ.MapManager(k=300)
    ctx = Context(P)
    est_h, _ = TJ.run(TJ.gpu_keyframe_fn(ctx), P, poses, odo, scans, 300, mm=host_mm)
    ctx.close()
    ctx = Context(P)
    dm = DeviceMapManager(capacity=4096, k=300, recent=200)
    est_d, _ = TJ.run_mapped(ctx, dm, P, poses, odo, scans)
    ctx.close()
    # the same keyframes on the same submaps: identical poses and maps
    for (Rh, th), (Rd, td) in zip(est_h, est_d):
        assert np.array_equal(np.asarray(Rh), np.asarray(Rd))
        assert np.array_equal(np.asarray(th), np.asarray(td))
    models, hits = dm.read()
    assert np.array_equal(models, host_mm.models)
    assert list(hits) == host_mm.hits
    assert dm.size()[2] == 0
    dm.close()


def test_mapped_keyframe_refuses_an_empty_submap():
    """A later keyframe whose submap is empty returns SLOAM_ERR_EMPTY_MAP
    (the reference's early return, sloamNode.cpp:199-203) and leaves the
    device map as it was."""
    import ctypes as C
    from sloam_gb300 import capi as A, synth
    from sloam_gb300.lib import Context, DeviceMapManager
    cfg = synth.C2
    forest, kfs = synth.scene(cfg, seed=0, n_kf=2)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1)
    ctx = Context(P)
    mapc = A.cylinders_from_array(forest.map_cylinders())
    kf0 = kfs[0]
    r = A.RunBuffers(P)
    ctx.check(ctx.L.sloam_keyframe(ctx.h, A.ptr(kf0.xyzi, C.c_float), len(kf0.xyzi),
                                   A.ptr(kf0.labels, C.c_uint8), None,
                                   C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), mapc,
                                   len(forest.radius), C.byref(r.s)))
    dm = DeviceMapManager(capacity=1024, k=100, recent=200)
    kf = kfs[1]
    r = A.RunBuffers(P)
    st = ctx.L.sloam_keyframe_mapped(ctx.h, dm.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                     A.ptr(kf.labels, C.c_uint8), None,
                                     C.byref(A.SE3.from_qt(*kf.pose_est_qt())), C.byref(r.s))
    assert st == A.SLOAM_ERR_EMPTY_MAP
    assert r.s.success == 0
    assert dm.size() == (0, 0, 0)
    dm.close()
    ctx.close()
