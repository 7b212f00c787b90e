"""The oracle's trust-region Levenberg-Marquardt pose solve (pose_solver 1;
the solver settings the reference gives Ceres, sloam.cpp:91-97, 149-155),
on the CPU: on the 64x2048 synthetic keyframe it lands on the same optimum
as the Gauss-Newton path (both minimise the same robust cost), moves the
pose towards the truth, and honours its iteration cap."""
import ctypes as C

import numpy as np
import pytest

from sloam_gb300 import capi as A, synth
from tests import helpers as H


def _second_pose(P, forest, kf):
    """First scan at the true pose, then the keyframe at its perturbed
    estimate through the oracle; returns (status, success, t, q)."""
    L = H.oracle()
    s = L.oracle_create(C.byref(P))
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    out = []
    for pose in (kf.pose_gt_qt(), kf.pose_est_qt()):
        r = A.RunBuffers(P)
        st = L.oracle_keyframe(s, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                               A.ptr(kf.labels, C.c_uint8), None,
                               C.byref(A.SE3.from_qt(*pose)), mapc, nm, C.byref(r.s))
        q, t = r.s.T_Map_Curr.qt()
        out.append((st, r.s.success, t, q))
    L.oracle_destroy(s)
    return out[1]


@pytest.mark.parametrize("two_step", [0, 1])
def test_lm_reaches_the_gn_optimum(two_step):
    cfg, forest, kfs = H.scene("C2")
    kf = kfs[0]
    res = {}
    for solver in (0, 1):
        P = synth.preset_params(cfg, two_step_optim=two_step, cyl_mode=1, pose_solver=solver)
        res[solver] = _second_pose(P, forest, kf)
    (st0, ok0, t0, q0), (st1, ok1, t1, q1) = res[0], res[1]
    assert st0 == st1 == 0 and ok0 and ok1
    assert np.abs(t1 - t0).max() < 10 * H.TOL_TRANS_M
    assert H.rot_angle(q0, q1) < 10 * H.TOL_ROT_RAD
    assert np.linalg.norm(t1 - kf.t_gt) < np.linalg.norm(kf.pose_est_qt()[1] - kf.t_gt)


def test_lm_iteration_cap():
    cfg, forest, kfs = H.scene("C2")
    kf = kfs[0]
    full = _second_pose(synth.preset_params(cfg, two_step_optim=0, cyl_mode=1,
                                            pose_solver=1), forest, kf)
    one = _second_pose(synth.preset_params(cfg, two_step_optim=0, cyl_mode=1, pose_solver=1,
                                           lm_max_iters=1), forest, kf)
    assert one[0] == 0 and np.isfinite(one[2]).all()
    # one step from the estimate is not yet the converged pose
    assert np.abs(one[2] - full[2]).max() > 10 * H.TOL_TRANS_M
