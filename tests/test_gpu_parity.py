"""GPU kernels vs the oracle through the C ABI, on the same inputs.

Bit-exact: pixel indices, range image, mask, ground list, tree cloud,
component labels, landmarks (ids, vertices, medians, radii, point lists),
plane bins, cylinder ids, RANSAC inlier counts, cylinder features, matches.
Within tolerance (FP64 oracle): plane / cylinder geometry (axis <= 1e-4 rad,
offset / radius <= 1e-4 m), pose (translation <= 1e-5 m, rotation <= 1e-6 rad).
"""
import ctypes as C

import numpy as np
import pytest

from sloam_gb300 import capi as A
from sloam_gb300 import synth
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sloam_gb300 import build
    build.build()


def make_ctx(P):
    from sloam_gb300.lib import Context
    return Context(P)


def assert_scan_equal(a, b):
    np.testing.assert_array_equal(a["px"], b["px"])
    np.testing.assert_array_equal(a["py"], b["py"])
    np.testing.assert_array_equal(a["range_image"].view(np.uint32), b["range_image"].view(np.uint32))
    np.testing.assert_array_equal(a["mask_out"], b["mask_out"])
    assert a["n_ground"] == b["n_ground"]
    n = a["n_ground"]
    np.testing.assert_array_equal(a["ground_idx"][:n], b["ground_idx"][:n])
    np.testing.assert_array_equal(a["tree_cloud"].view(np.uint32), b["tree_cloud"].view(np.uint32))


# ------------------------------------------------------------------ a1/a2
@pytest.mark.parametrize("name", ["C1", "C2"])
@pytest.mark.parametrize("destagger", [0, 1])
def test_projection_point_labels(name, destagger):
    cfg, forest, kfs = H.scene(name)
    P = synth.preset_params(cfg, do_destagger=destagger)
    ctx = make_ctx(P)
    kf = kfs[0]
    o = H.oracle_project(P, kf.xyzi, labels=kf.labels)
    g = H.gpu_project(ctx, kf.xyzi, labels=kf.labels)
    assert_scan_equal(o, g)


def test_projection_mask_image_and_edge_points():
    cfg, forest, kfs = H.scene("C2")
    P = synth.preset_params(cfg)
    ctx = make_ctx(P)
    xyzi = kfs[0].xyzi.copy()
    rng = np.random.default_rng(3)
    n = len(xyzi)
    # edge cases: zero points, signed zeros on the axes, tiny and huge coordinates
    idx = rng.choice(n, 64, replace=False)
    xyzi[idx[0:8], :3] = 0.0
    xyzi[idx[8:16], 1] = -0.0
    xyzi[idx[8:16], 0] = -5.0
    xyzi[idx[16:24], 1] = 0.0
    xyzi[idx[16:24], 0] = -5.0
    xyzi[idx[24:32], :3] = 1e-30
    xyzi[idx[32:40], :3] = [1e19, -1e19, 3e18]
    xyzi[idx[40:48], 0] = np.nan
    xyzi[idx[48:56], 2] = 100.0   # beyond the vertical field of view
    xyzi[idx[56:64], 2] = -100.0
    labels = kfs[0].labels
    o = H.oracle_project(P, xyzi, labels=labels)
    g = H.gpu_project(ctx, xyzi, labels=labels)
    assert_scan_equal(o, g)
    # mask-image mode: the network-style per-pixel mask
    mask = o["mask_out"].copy()
    o2 = H.oracle_project(P, xyzi, mask=mask)
    g2 = H.gpu_project(ctx, xyzi, mask=mask)
    assert_scan_equal(o2, g2)


def test_projection_random_directions_many_scans():
    """Uniform random directions hit column/row boundaries everywhere."""
    P = A.default_params(img_w=2048, img_h=64)
    ctx = make_ctx(P)
    rng = np.random.default_rng(11)
    for _ in range(4):
        n = P.img_w * P.img_h
        v = rng.normal(size=(n, 3)).astype(np.float32)
        r = rng.uniform(0.5, 40, n).astype(np.float32)
        xyzi = np.zeros((n, 4), np.float32)
        xyzi[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None]
        lab = rng.choice(np.array([0, 1, 255], np.uint8), n)
        o = H.oracle_project(P, xyzi, labels=lab)
        g = H.gpu_project(ctx, xyzi, labels=lab)
        assert_scan_equal(o, g)


# ------------------------------------------------------------------ a3-a5
@pytest.mark.parametrize("seq", ["still", "moving"])
@pytest.mark.parametrize("t", ["t0", "t1"])
def test_trellis_reference_clouds(seq, t):
    cloud, h, w = H.golden_tree_cloud(seq, t)
    P = A.default_params()
    ctx = make_ctx(P)
    lo, labo, nco = H.oracle_trellis(P, cloud, h, w)
    lg, labg, ncg = H.gpu_trellis(ctx, cloud, h, w)
    assert nco == ncg
    np.testing.assert_array_equal(labo, labg)
    H.landmarks_equal_exact(lo, lg)


def test_trellis_known_answer_on_gpu():
    """The reference's stored Trellis output, reproduced by the GPU."""
    cloud, h, w = H.golden_tree_cloud("still", "t0")
    ctx = make_ctx(A.default_params())
    lg, _, _ = H.gpu_trellis(ctx, cloud, h, w)
    ref = H.golden_landmarks("still", "t0")
    trees = lg.to_trees()
    assert [t[0]["tree_id"] for t in trees] == [t[0]["tree_id"] for t in ref]
    assert [len(t) for t in trees] == [len(t) for t in ref]
    for tr, rt in zip(trees, ref):
        for v, rv in zip(tr, rt):
            np.testing.assert_allclose(v["xyz"], rv["xyz"], atol=2e-6, rtol=0)
            assert abs(0.5 * v["radius"] - rv["radius"]) < 2e-6
            np.testing.assert_allclose(v["points"][:, :3], rv["points"][:, :3], atol=2e-6, rtol=0)


@pytest.mark.parametrize("name", ["C1", "C2"])
def test_trellis_synthetic(name):
    cfg, forest, kfs = H.scene(name)
    P = synth.preset_params(cfg)
    ctx = make_ctx(P)
    o = H.oracle_project(P, kfs[0].xyzi, labels=kfs[0].labels)
    cloud = o["tree_cloud"]
    lo, labo, nco = H.oracle_trellis(P, cloud, P.img_h, P.img_w)
    lg, labg, ncg = H.gpu_trellis(ctx, cloud, P.img_h, P.img_w)
    assert lo.s.n_landmarks > 0
    assert nco == ncg
    np.testing.assert_array_equal(labo, labg)
    H.landmarks_equal_exact(lo, lg)


def test_trellis_empty_cloud():
    P = A.default_params()
    ctx = make_ctx(P)
    cloud = np.full((P.img_w * P.img_h, 4), np.nan, np.float32)
    lg, labg, ncg = H.gpu_trellis(ctx, cloud, P.img_h, P.img_w)
    assert ncg == 0 and lg.s.n_landmarks == 0
    assert (labg == 0xFFFFFFFF).all()


# ------------------------------------------------------------------ a6-a8
def core_params(two_step, cyl_mode=0):
    from tests.test_oracle_reference import core_params as cp
    p = cp(two_step)
    p.cyl_mode = cyl_mode
    return p


@pytest.mark.parametrize("cyl_mode", [0, 1])
def test_models_reference_landmarks(cyl_mode):
    P = core_params(1, cyl_mode)
    ctx = make_ctx(P)
    lb = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t0", resize_points=5))
    g0 = H.golden_ground("t0")
    I = A.SE3.identity()
    mo = H.oracle_models(P, I, g0, lb)
    mg = H.gpu_models(ctx, I, g0, lb)
    assert mo.s.n_planes > 0 and mo.s.n_cylinders > 0
    H.compare_models(mo, mg)


@pytest.mark.parametrize("cyl_mode", [0, 1])
def test_models_synthetic_c2(cyl_mode):
    cfg, forest, kfs = H.scene("C2")
    P = synth.preset_params(cfg, cyl_mode=cyl_mode)
    ctx = make_ctx(P)
    kf = kfs[0]
    o = H.oracle_project(P, kf.xyzi, labels=kf.labels)
    ground = np.ascontiguousarray(kf.xyzi[o["ground_idx"][:o["n_ground"]]])
    lo, _, _ = H.oracle_trellis(P, o["tree_cloud"], P.img_h, P.img_w)
    pose = A.SE3.from_qt(*kf.pose_est_qt())
    mo = H.oracle_models(P, pose, ground, lo)
    mg = H.gpu_models(ctx, pose, ground, lo)
    assert mo.s.n_cylinders > 10
    H.compare_models(mo, mg)


# --------------------------------------------------------------- a9-a11
def gpu_run_pair(ctx):
    L = ctx.L
    lm0 = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t0", resize_points=5))
    lm1 = A.LandmarkBuffers.from_trees(H.golden_landmarks("still", "t1", resize_points=5))
    g0, g1 = H.golden_ground("t0"), H.golden_ground("t1")
    I = A.SE3.identity()
    r0 = A.RunBuffers(ctx.params)
    st0 = L.sloam_run(ctx.h, C.byref(I), A.ptr(g0, C.c_float), len(g0), C.byref(lm0.s), None, 0,
                      C.byref(r0.s))
    r0.refresh()
    m = A.cylinders_from_array(r0.m.cyl_array())
    r1 = A.RunBuffers(ctx.params)
    st1 = L.sloam_run(ctx.h, C.byref(I), A.ptr(g1, C.c_float), len(g1), C.byref(lm1.s), m,
                      r0.s.models.n_cylinders, C.byref(r1.s))
    r1.refresh()
    return st0, r0, st1, r1


def compare_runs(ro, rg, pose_tol=1.0):
    """Statuses, checks, match counts and indices exactly; models and pose
    within the tolerances times pose_tol (the models are returned in the map
    frame, moved by the estimated pose, so they share its tolerance)."""
    assert ro.s.success == rg.s.success
    assert ro.s.n_tree_matches == rg.s.n_tree_matches
    assert ro.s.n_plane_matches == rg.s.n_plane_matches
    assert ro.s.tree_check == rg.s.tree_check and ro.s.ground_check == rg.s.ground_check
    H.compare_models(ro.m, rg.m, tol_scale=pose_tol)
    n = ro.s.models.n_cylinders
    np.testing.assert_array_equal(ro.matches[:n], rg.matches[:n])
    qo, to = ro.s.T_Map_Curr.qt()
    qg, tg = rg.s.T_Map_Curr.qt()
    assert np.abs(to - tg).max() < H.TOL_TRANS_M * pose_tol, (to, tg)
    assert H.rot_angle(qo, qg) < H.TOL_ROT_RAD * pose_tol, (qo, qg)


@pytest.mark.parametrize("two_step,solver", [(0, 0), (1, 0), (0, 1)])
def test_run_reference_pair(two_step, solver):
    from tests.test_oracle_reference import oracle_run_pair
    P = core_params(two_step)
    P.pose_solver = solver
    ctx = make_ctx(P)
    st0, r0, st1, r1 = gpu_run_pair(ctx)
    so0, ro0, so1, ro1 = oracle_run_pair(P)
    assert (st0, st1) == (so0, so1) == (0, 0)
    compare_runs(ro0, r0)
    compare_runs(ro1, r1)
    # core_test.cpp properties on the GPU result
    assert r0.s.models.n_cylinders > 0 and r0.s.models.n_planes > 0
    assert r1.s.success and (r1.matches[:r1.s.models.n_cylinders] != -1).any()
    # PoseOptimization (core_test.cpp:177), unrelaxed: |T_Delta.t| < 0.1 m
    assert np.linalg.norm(np.array(r1.s.T_Delta.t[:])) < 0.1


def keyframe_pair(P, forest, kf, run):
    """first scan at the true pose (defines map-frame planes), then the
    keyframe at the perturbed estimate; returns both outputs."""
    mapc = A.cylinders_from_array(forest.map_cylinders())
    gt = A.SE3.from_qt(*kf.pose_gt_qt())
    est = A.SE3.from_qt(*kf.pose_est_qt())
    r0, r1 = A.RunBuffers(P), A.RunBuffers(P)
    s0 = run(kf, gt, mapc, len(forest.radius), r0)
    s1 = run(kf, est, mapc, len(forest.radius), r1)
    r0.refresh()
    r1.refresh()
    return s0, r0, s1, r1


@pytest.mark.parametrize("two_step,cyl_mode", [(0, 1), (1, 0), (0, 0)])
def test_keyframe_synthetic_c2(two_step, cyl_mode):
    cfg, forest, kfs = H.scene("C2")
    P = synth.preset_params(cfg, two_step_optim=two_step, cyl_mode=cyl_mode)
    ctx = make_ctx(P)
    L = H.oracle()
    os_ = L.oracle_create(C.byref(P))

    def run_o(kf, pose, m, nm, r):
        return L.oracle_keyframe(os_, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                 A.ptr(kf.labels, C.c_uint8), None, C.byref(pose), m, nm,
                                 C.byref(r.s))

    def run_g(kf, pose, m, nm, r):
        return ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                    A.ptr(kf.labels, C.c_uint8), None, C.byref(pose), m, nm,
                                    C.byref(r.s))

    so0, ro0, so1, ro1 = keyframe_pair(P, forest, kfs[0], run_o)
    sg0, rg0, sg1, rg1 = keyframe_pair(P, forest, kfs[0], run_g)
    L.oracle_destroy(os_)
    assert (so0, so1) == (sg0, sg1)
    compare_runs(ro0, rg0)
    compare_runs(ro1, rg1)
    # the pose moved towards the truth
    q, t = rg1.s.T_Map_Curr.qt()
    assert np.linalg.norm(t - kfs[0].t_gt) < 0.1


@pytest.mark.parametrize("seed", [0, 2, 3])
@pytest.mark.parametrize("two_step,cyl_mode", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_keyframe_synthetic_c1(seed, two_step, cyl_mode):
    """16x1024 keyframes (ground slope U(0, 10 deg), 20 trunks, 64
    hypotheses per tree), the first scan at the true pose then the keyframe
    at its estimate, GPU against the oracle in both cylinder modes and both
    pose modes.  Sixteen beams leave a few trees per scan: seed 0 fits 3
    cylinders on 3 and 2 planes, seed 2 finds no cylinder (the second
    keyframe ends in SLOAM_ERR_NO_MODELS, sloam.cpp:481-485), seed 3 none on
    the first scan and one on the second.  Too few tree features for the
    pose checks (sloam.cpp:497-499) keep the estimate as it was; the two
    sides agree on every outcome."""
    cfg = synth.C1
    forest, kfs = synth.scene(cfg, seed=seed, n_kf=1)
    P = synth.preset_params(cfg, two_step_optim=two_step, cyl_mode=cyl_mode, cyl_hypotheses=64)
    ctx = make_ctx(P)
    L = H.oracle()
    os_ = L.oracle_create(C.byref(P))

    def run_o(kf, pose, m, nm, r):
        return L.oracle_keyframe(os_, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                 A.ptr(kf.labels, C.c_uint8), None, C.byref(pose), m, nm,
                                 C.byref(r.s))

    def run_g(kf, pose, m, nm, r):
        return ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                    A.ptr(kf.labels, C.c_uint8), None, C.byref(pose), m, nm,
                                    C.byref(r.s))

    so0, ro0, so1, ro1 = keyframe_pair(P, forest, kfs[0], run_o)
    sg0, rg0, sg1, rg1 = keyframe_pair(P, forest, kfs[0], run_g)
    L.oracle_destroy(os_)
    ctx.close()
    assert (so0, so1) == (sg0, sg1)
    compare_runs(ro0, rg0)
    if so1 == 0:
        compare_runs(ro1, rg1)
    else:
        assert so1 == A.SLOAM_ERR_NO_MODELS
        assert ro1.s.models.n_cylinders == rg1.s.models.n_cylinders == 0


@pytest.mark.parametrize("two_step", [0, 1])
def test_keyframe_lm_c2(two_step):
    """pose_solver 1 (trust-region Levenberg-Marquardt with the reference's
    Ceres settings) on the GPU against the oracle's: the same models and
    matches, poses within 5e-5 m / 5e-6 rad.  The LM stops when a step
    changes the cost by at most 1e-6 of it (Ceres' function tolerance); the
    GPU sums FP32 residuals, whose rounding is of that order, so the two
    sides can stop one step apart near the optimum (measured up to 1.6e-5 m;
    the GN pose, with a fixed iteration count, keeps 1e-5 m).  The LM optimum
    and the 10-iteration GN pose agree within 10x the GN tolerance (measured
    2e-5 m on the two-step pose)."""
    cfg, forest, kfs = H.scene("C2")
    L = H.oracle()
    out = {}
    for solver in (0, 1):
        P = synth.preset_params(cfg, two_step_optim=two_step, cyl_mode=1, pose_solver=solver)
        os_ = L.oracle_create(C.byref(P))

        def run_o(kf, pose, m, nm, r):
            return L.oracle_keyframe(os_, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                     A.ptr(kf.labels, C.c_uint8), None, C.byref(pose), m, nm,
                                     C.byref(r.s))
        out[solver, "o"] = keyframe_pair(P, forest, kfs[0], run_o)
        L.oracle_destroy(os_)
        if solver == 1:
            ctx = make_ctx(P)

            def run_g(kf, pose, m, nm, r):
                return ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                            A.ptr(kf.labels, C.c_uint8), None, C.byref(pose),
                                            m, nm, C.byref(r.s))
            out[solver, "g"] = keyframe_pair(P, forest, kfs[0], run_g)
            ctx.close()
    so0, ro0, so1, ro1 = out[1, "o"]
    sg0, rg0, sg1, rg1 = out[1, "g"]
    assert (so0, so1) == (sg0, sg1)
    compare_runs(ro0, rg0)
    _, t_o = ro1.s.T_Map_Curr.qt()
    _, t_g = rg1.s.T_Map_Curr.qt()
    _, t_gn = out[0, "o"][3].s.T_Map_Curr.qt()
    print("LM gpu-oracle", np.abs(t_g - t_o).max(), "LM-GN", np.abs(t_o - t_gn).max())
    compare_runs(ro1, rg1, pose_tol=5.0)
    assert np.abs(t_o - t_gn).max() < 10 * H.TOL_TRANS_M
    assert np.linalg.norm(t_g - kfs[0].t_gt) < 0.1


def _first_scan(ctx, P, kf0, mapc, n_map):
    r = A.RunBuffers(P)
    ctx.check(ctx.L.sloam_keyframe(ctx.h, A.ptr(kf0.xyzi, C.c_float), len(kf0.xyzi),
                                   A.ptr(kf0.labels, C.c_uint8), None,
                                   C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), mapc, n_map,
                                   C.byref(r.s)))


def _single_results(P, kfs, mapc, n_map):
    """Each keyframe alone through sloam_keyframe on a fresh context whose
    first scan is keyframe 0 at its true pose: (q, t, n_cylinders, success)."""
    out = []
    for kf in kfs:
        ctx = make_ctx(P)
        _first_scan(ctx, P, kfs[0], mapc, n_map)
        r1 = A.RunBuffers(P)
        st = ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                  A.ptr(kf.labels, C.c_uint8), None,
                                  C.byref(A.SE3.from_qt(*kf.pose_est_qt())), mapc, n_map,
                                  C.byref(r1.s))
        r1.refresh()
        q, t = r1.s.T_Map_Curr.qt()
        out.append((q, t, r1.s.models.n_cylinders, 1 if st == 0 and r1.s.success else 0))
        ctx.close()
    return out


def _check_batch(po, succ, ncyl, order, ref):
    for k, j in enumerate(order):
        q, t, nc, ok = ref[j]
        np.testing.assert_array_equal(po[k, :4], q)
        np.testing.assert_array_equal(po[k, 4:], t)
        assert int(ncyl[k]) == nc
        assert int(succ[k]) == ok


@pytest.mark.parametrize("destagger", [0, 1])
def test_keyframes_batches_match_single(destagger):
    """Batches through the device and the host entry points: 37 keyframes
    (several batch projection launches, the last one partial) over five
    slots, each result bit-identical to the keyframe run alone.  The batch
    keeps the tree cloud and the ground list as views of the scan (tree
    flags, ground indices); the keyframe alone materialises them."""
    import torch
    cfg, forest, kfs = H.scene("C2", seed=0, n_kf=3)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1, do_destagger=destagger)
    P.batch_slots = 5
    mapa = forest.map_cylinders()
    mapc = A.cylinders_from_array(mapa)
    nm = len(mapa)
    ref = _single_results(P, kfs, mapc, nm)
    ctx = make_ctx(P)
    _first_scan(ctx, P, kfs[0], mapc, nm)
    B = 37
    order = [k % len(kfs) for k in range(B)]
    n = len(kfs[0].xyzi)
    xs = np.stack([kfs[j].xyzi for j in order])
    ls = np.stack([kfs[j].labels for j in order])
    poses = (A.SE3 * B)(*[A.SE3.from_qt(*kfs[j].pose_est_qt()) for j in order])
    dx = torch.from_numpy(xs).cuda()
    dl = torch.from_numpy(ls).cuda()
    dm = torch.from_numpy(np.frombuffer(bytes(mapc), np.uint8).copy()).cuda()
    pose_out = torch.zeros(B * 7, dtype=torch.float64, device="cuda")
    succ = torch.zeros(B, dtype=torch.int32, device="cuda")
    ncyl = torch.zeros(B, dtype=torch.int32, device="cuda")
    for _ in range(2):  # the second call reuses the batch buffers and graphs
        pose_out.zero_()
        ctx.check(ctx.L.sloam_keyframes_device(ctx.h, dx.data_ptr(), n, B, dl.data_ptr(), poses,
                                               dm.data_ptr(), nm, pose_out.data_ptr(),
                                               succ.data_ptr(), ncyl.data_ptr()))
        torch.cuda.synchronize()
        _check_batch(pose_out.cpu().numpy().reshape(-1, 7), succ.cpu(), ncyl.cpu(), order, ref)
    h_pose = np.zeros(B * 7, np.float64)
    h_succ = np.zeros(B, np.int32)
    h_ncyl = np.zeros(B, np.int32)
    ctx.check(ctx.L.sloam_keyframes_host(ctx.h, A.ptr(xs, C.c_float), n, B,
                                         A.ptr(ls, C.c_uint8), poses, mapc, nm,
                                         h_pose.ctypes.data, h_succ.ctypes.data,
                                         h_ncyl.ctypes.data))
    _check_batch(h_pose.reshape(-1, 7), h_succ, h_ncyl, order, ref)
    ms, nch, nkf = C.c_float(), C.c_int32(), C.c_int32()
    ctx.check(ctx.L.sloam_frontend_time(ctx.h, C.byref(ms), C.byref(nch), C.byref(nkf)))
    assert nkf.value == B and nch.value >= 2 and ms.value > 0
    ctx.close()


def _scan_out_equal(g, o, n_ground):
    np.testing.assert_array_equal(g["range_image"].view(np.uint32), o["range_image"].view(np.uint32))
    np.testing.assert_array_equal(g["mask_out"], o["mask_out"])
    assert n_ground == o["n_ground"]
    np.testing.assert_array_equal(g["ground_idx"][:n_ground], o["ground_idx"][:n_ground])
    np.testing.assert_array_equal(g["tree_cloud"].view(np.uint32), o["tree_cloud"].view(np.uint32))


@pytest.mark.parametrize("destagger", [0, 1])
def test_batch_projection_matches_oracle(destagger):
    """The batch projection (the resident projection grid, the label pass
    and the ordered ground compaction, the pixel keys re-armed chunk by
    chunk): 37 keyframes through the device entry point (one launch group)
    twice, then through the host entry point (chunks of 8 on two
    alternating scratch sets, a chunk's labels overlapping the next chunk's
    projection), every keyframe's range image, mask, ground list and
    organised tree cloud bit-identical to the oracle's projection of its
    scan."""
    import torch
    cfg, forest, kfs = H.scene("C2", seed=3, n_kf=3)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1, do_destagger=destagger)
    P.batch_slots = 3
    mapa = forest.map_cylinders()
    mapc = A.cylinders_from_array(mapa)
    nm = len(mapa)
    ref = [H.oracle_project(P, kf.xyzi, labels=kf.labels) for kf in kfs]
    ctx = make_ctx(P)
    _first_scan(ctx, P, kfs[0], mapc, nm)
    B = 37
    order = [(5 * k) % len(kfs) for k in range(B)]
    n = len(kfs[0].xyzi)
    xs = np.stack([kfs[j].xyzi for j in order])
    ls = np.stack([kfs[j].labels for j in order])
    poses = (A.SE3 * B)(*[A.SE3.from_qt(*kfs[j].pose_est_qt()) for j in order])
    dx = torch.from_numpy(xs).cuda()
    dl = torch.from_numpy(ls).cuda()
    dm = torch.from_numpy(np.frombuffer(bytes(mapc), np.uint8).copy()).cuda()
    pose_out = torch.zeros(B * 7, dtype=torch.float64, device="cuda")
    succ = torch.zeros(B, dtype=torch.int32, device="cuda")
    ncyl = torch.zeros(B, dtype=torch.int32, device="cuda")

    def check_all():
        for k, j in enumerate(order):
            b, s = H.scan_buffers(n, P.img_h, P.img_w)
            s.px = None
            s.py = None
            ctx.check(ctx.L.sloam_batch_scan_out(ctx.h, k, C.byref(s)))
            _scan_out_equal(b, ref[j], s.n_ground)

    for _ in range(2):
        ctx.check(ctx.L.sloam_keyframes_device(ctx.h, dx.data_ptr(), n, B, dl.data_ptr(), poses,
                                               dm.data_ptr(), nm, pose_out.data_ptr(),
                                               succ.data_ptr(), ncyl.data_ptr()))
        torch.cuda.synchronize()
        check_all()
    h_pose = np.zeros(B * 7, np.float64)
    h_succ = np.zeros(B, np.int32)
    h_ncyl = np.zeros(B, np.int32)
    ctx.check(ctx.L.sloam_keyframes_host(ctx.h, A.ptr(xs, C.c_float), n, B,
                                         A.ptr(ls, C.c_uint8), poses, mapc, nm,
                                         h_pose.ctypes.data, h_succ.ctypes.data,
                                         h_ncyl.ctypes.data))
    check_all()
    # px / py are not kept for batch keyframes; a keyframe past the batch
    b, s = H.scan_buffers(n, P.img_h, P.img_w)
    assert ctx.L.sloam_batch_scan_out(ctx.h, 0, C.byref(s)) == A.SLOAM_ERR_ARG
    s.px = None
    s.py = None
    assert ctx.L.sloam_batch_scan_out(ctx.h, B, C.byref(s)) == A.SLOAM_ERR_ARG
    ctx.close()


def test_cc_union_limit_runs_out_and_context_recovers():
    """The bounded union loop of the connected components gives up: with a
    retry limit of 0 every union that is needed fails at once, the kernels
    record it and return, the keyframe ends with SLOAM_ERR_TIMEOUT and its
    message, and the same context then runs the keyframe normally (the
    oracle's result) once the default limit is back."""
    cfg, forest, kfs = H.scene("C2")
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1)
    ctx = make_ctx(P)
    kf = kfs[0]
    mapc = A.cylinders_from_array(forest.map_cylinders())
    gt = A.SE3.from_qt(*kf.pose_gt_qt())

    def run():
        r = A.RunBuffers(P)
        st = ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                  A.ptr(kf.labels, C.c_uint8), None, C.byref(gt), mapc,
                                  len(forest.radius), C.byref(r.s))
        r.refresh()
        return st, r

    assert ctx.L.sloam_set_cc_iter_limit(ctx.h, 0) == 0
    st, _ = run()
    assert st == A.SLOAM_ERR_TIMEOUT
    assert "iteration limit" in ctx.error()
    assert ctx.L.sloam_set_cc_iter_limit(ctx.h, -1) == 0
    assert ctx.L.sloam_reset(ctx.h) == 0
    st, rg = run()
    assert st == 0 and rg.s.models.n_cylinders > 10
    L = H.oracle()
    os_ = L.oracle_create(C.byref(P))
    ro = A.RunBuffers(P)
    so = L.oracle_keyframe(os_, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                           A.ptr(kf.labels, C.c_uint8), None, C.byref(gt), mapc,
                           len(forest.radius), C.byref(ro.s))
    ro.refresh()
    L.oracle_destroy(os_)
    assert so == 0
    compare_runs(ro, rg)
    ctx.close()
