"""The uneven batch (64x2048 keyframes with 20-400 trees and clusters of a
few to ~20k points): per-keyframe parity with the oracle, and a batch of
keyframes of very different sizes through one batch call equal to the same
keyframes run one by one."""
import ctypes as C

import numpy as np
import pytest

from sloam_gb300 import capi as A
from sloam_gb300 import synth
from tests import helpers as H

COUNTS = [20, 400, 60, 150, 300, 35]


def _scene():
    return H.c3_scene(tuple(COUNTS))


def test_c3_generator_spans_the_sizes():
    forest, kfs, counts = _scene()
    assert counts == COUNTS
    sizes = []
    for kf in kfs:
        th = kf.tree_hit
        _, cnt = np.unique(th[th >= 0], return_counts=True)
        sizes.append(cnt)
    allc = np.concatenate(sizes)
    assert allc.max() > 9000 and allc.min() < 50
    # every keyframe sees only its own cell
    assert len(forest.radius) == sum(COUNTS)


def test_c3_drawn_counts_in_range():
    f, kfs, counts = synth.c3_scene(3, n_kf=8)
    assert len(kfs) == 8 and all(20 <= c <= 400 for c in counts)
    assert len(f.radius) == sum(counts)


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(COUNTS)))
def test_c3_keyframe_matches_oracle(k):
    from tests.test_gpu_parity import compare_runs, keyframe_pair, make_ctx
    forest, kfs, _ = _scene()
    P = synth.c3_params(forest, two_step_optim=0, cyl_mode=1)
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

    so0, ro0, so1, ro1 = keyframe_pair(P, forest, kfs[k], run_o)
    sg0, rg0, sg1, rg1 = keyframe_pair(P, forest, kfs[k], run_g)
    L.oracle_destroy(os_)
    ctx.close()
    assert (so0, so1) == (sg0, sg1)
    compare_runs(ro0, rg0)
    compare_runs(ro1, rg1)


@pytest.mark.gpu
def test_c3_batch_matches_single():
    import torch
    from tests.test_gpu_parity import _check_batch, _first_scan, _single_results, make_ctx
    forest, kfs, _ = _scene()
    P = synth.c3_params(forest, two_step_optim=0, cyl_mode=1)
    P.batch_slots = 4
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    ref = _single_results(P, kfs, mapc, nm)
    ctx = make_ctx(P)
    _first_scan(ctx, P, kfs[0], mapc, nm)
    B = len(kfs)
    n = len(kfs[0].xyzi)
    dx = torch.from_numpy(np.stack([kf.xyzi for kf in kfs])).cuda()
    dl = torch.from_numpy(np.stack([kf.labels for kf in kfs])).cuda()
    dm = torch.from_numpy(np.frombuffer(bytes(mapc), np.uint8).copy()).cuda()
    poses = (A.SE3 * B)(*[A.SE3.from_qt(*kf.pose_est_qt()) for kf in kfs])
    pose_out = torch.zeros(B * 7, dtype=torch.float64, device="cuda")
    succ = torch.zeros(B, dtype=torch.int32, device="cuda")
    ncyl = torch.zeros(B, dtype=torch.int32, device="cuda")
    ctx.check(ctx.L.sloam_keyframes_device(ctx.h, dx.data_ptr(), n, B, dl.data_ptr(), poses,
                                           dm.data_ptr(), nm, pose_out.data_ptr(),
                                           succ.data_ptr(), ncyl.data_ptr()))
    torch.cuda.synchronize()
    _check_batch(pose_out.cpu().numpy().reshape(-1, 7), succ.cpu(), ncyl.cpu(), list(range(B)), ref)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("chunk,tile,blocks", [(512, 64, 8), (1024, 1024, 300), (256, 128, 1)])
def test_c3_queue_shapes_bit_identical(chunk, tile, blocks):
    """The work queue's shape (points per item, hypotheses staged per pass,
    persistent blocks: what the autotuner chooses) changes how the work is
    cut, not the result: every keyframe's cylinders (inlier counts, fits),
    matches and pose are bit-identical to the default shape's."""
    from tests.test_gpu_parity import make_ctx
    forest, kfs, _ = _scene()
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    out = {}
    for shape in ((256, 256, 0), (chunk, tile, blocks)):
        P = synth.c3_params(forest, two_step_optim=0, cyl_mode=1)
        P.cyl_chunk_points, P.cyl_hyp_tile, P.cyl_queue_blocks = shape
        ctx = make_ctx(P)
        res = []
        for k in (1, 3, 4):  # 400, 150 and 300 trees
            kf = kfs[k]
            rr = []
            for pose in (A.SE3.from_qt(*kf.pose_gt_qt()), A.SE3.from_qt(*kf.pose_est_qt())):
                r = A.RunBuffers(P)
                ctx.check(ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                               A.ptr(kf.labels, C.c_uint8), None, C.byref(pose),
                                               mapc, nm, C.byref(r.s)))
                r.refresh()
                n = r.s.models.n_cylinders
                q, t = r.s.T_Map_Curr.qt()
                rr.append((r.m.cyl_array()[:n].copy(), r.m.cyl_inliers[:n].copy(),
                           r.matches[:n].copy(), q, t))
            ctx.check(ctx.L.sloam_reset(ctx.h))
            res.append(rr)
        ctx.close()
        out[shape] = res
    a, b = out[(256, 256, 0)], out[(chunk, tile, blocks)]
    for ra, rb in zip(a, b):
        for xa, xb in zip(ra, rb):
            assert len(xa[0]) > 10
            for u, v in zip(xa, xb):
                np.testing.assert_array_equal(u, v)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [0, 4])
def test_c3_trellis_wide_rows_match_oracle(k):
    """Trellis of the uneven scenes whose near trunks give component rows of
    more than 256 points (284 and 294) (the block-per-row vertex
    kernel): component labels and landmarks (vertex medians, radii, kept
    points in order) bit-identical to the oracle's."""
    from tests.test_gpu_parity import make_ctx
    forest, kfs, _ = _scene()
    P = synth.c3_params(forest, two_step_optim=0, cyl_mode=1)
    kf = kfs[k]
    o = H.oracle_project(P, kf.xyzi, labels=kf.labels)
    cloud = o["tree_cloud"]
    lo, labo, nco = H.oracle_trellis(P, cloud, P.img_h, P.img_w)
    # some (component, row) holds more than 256 points
    lab = labo.reshape(P.img_h, P.img_w)
    widest = 0
    for r in range(P.img_h):
        row = lab[r][lab[r] != 0xFFFFFFFF]
        if len(row):
            widest = max(widest, np.unique(row, return_counts=True)[1].max())
    assert widest > 256
    ctx = make_ctx(P)
    lg, labg, ncg = H.gpu_trellis(ctx, cloud, P.img_h, P.img_w)
    assert nco == ncg
    np.testing.assert_array_equal(labo, labg)
    H.landmarks_equal_exact(lo, lg)
