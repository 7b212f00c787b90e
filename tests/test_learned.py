"""The learned-proposal cylinder mode (cyl_mode 2): network proposals scored
by inlier counts, RANSAC fallback, LS refinement.  It has no reference
counterpart, so it is checked against the generator's true trunks, side by
side with the plain point RANSAC (cyl_mode 1), and for batch/single
identity."""
import ctypes as C

import numpy as np
import pytest

from sloam_gb300 import capi as A
from sloam_gb300 import proposal, synth
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _ctx(P, weights=True):
    from sloam_gb300.lib import Context
    ctx = Context(P)
    if weights:
        ctx.set_proposal_weights(proposal.load_weights())
    return ctx


def _keyframe_errors(mode, n_kf=4):
    from tests.test_gpu_parity import keyframe_pair
    cfg, forest, kfs = H.scene("C2", seed=0, n_kf=n_kf)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=mode)
    ctx = _ctx(P, weights=(mode == 2))
    angs, rerrs, ok = [], [], []

    def run_g(kf, pose, m, nm, r):
        return ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                    A.ptr(kf.labels, C.c_uint8), None, C.byref(pose), m, nm,
                                    C.byref(r.s))
    for kf in kfs:
        s0, r0, s1, r1 = keyframe_pair(P, forest, kf, run_g)
        a, e = synth.cylinder_errors(forest, r1.m.cyl_array())
        angs.append(a)
        rerrs.append(e)
        ok.append(s1 == 0 and r1.s.success)
    ctx.close()
    return np.concatenate(angs), np.concatenate(rerrs), ok


def test_mode2_refuses_keyframes_without_weights():
    cfg, forest, kfs = H.scene("C2")
    P = synth.preset_params(cfg, cyl_mode=2)
    ctx = _ctx(P, weights=False)
    kf = kfs[0]
    r = A.RunBuffers(P)
    mapc = A.cylinders_from_array(forest.map_cylinders())
    st = ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                              A.ptr(kf.labels, C.c_uint8), None,
                              C.byref(A.SE3.from_qt(*kf.pose_gt_qt())), mapc, len(mapc),
                              C.byref(r.s))
    assert st == A.SLOAM_ERR_ARG and "proposal" in ctx.error()
    ctx.close()


def test_learned_mode_matches_plain_accuracy():
    a1, e1, ok1 = _keyframe_errors(1)
    a2, e2, ok2 = _keyframe_errors(2)
    print(f"plain: {len(a1)} trees, median axis {np.median(a1):.3f} deg, radius "
          f"{100 * np.median(e1):.2f} cm; learned: {len(a2)} trees, median axis "
          f"{np.median(a2):.3f} deg, radius {100 * np.median(e2):.2f} cm")
    assert all(ok2)
    assert len(a2) >= 0.9 * len(a1)
    # the benchmark's accuracy bound (median axis <= 0.5 deg, radius <= 1 cm)
    assert np.median(a2) <= 0.5 and np.median(e2) <= 0.01
    assert np.median(a2) <= np.median(a1) + 0.1 and np.median(e2) <= np.median(e1) + 0.003


def test_learned_batch_matches_single():
    import torch
    from tests.test_gpu_parity import _check_batch, _first_scan, make_ctx
    cfg, forest, kfs = H.scene("C2", seed=0, n_kf=3)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=2)
    P.batch_slots = 3
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    ref = []
    for kf in kfs:
        ctx = _ctx(P)
        _first_scan(ctx, P, kfs[0], mapc, nm)
        r1 = A.RunBuffers(P)
        st = ctx.L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                                  A.ptr(kf.labels, C.c_uint8), None,
                                  C.byref(A.SE3.from_qt(*kf.pose_est_qt())), mapc, nm,
                                  C.byref(r1.s))
        r1.refresh()
        q, t = r1.s.T_Map_Curr.qt()
        ref.append((q, t, r1.s.models.n_cylinders, 1 if st == 0 and r1.s.success else 0))
        ctx.close()
    ctx = _ctx(P)
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
