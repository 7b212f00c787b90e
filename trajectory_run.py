#!/usr/bin/env python3
"""Long-trajectory run (benchmark configuration 5): drift against ground
truth of the GPU path (plain RANSAC, learned proposals, and the plain path
with the map manager on the GPU) and of the CPU restatement of the reference
(the oracle), over the same seeded scene.

    python trajectory_run.py --kf 200 --h 128 --w 2048 [--out FILE]

200 keyframes of 128x2048, 1 m per keyframe, yaw rate at most 15 deg per
keyframe, a 1 000-tree forest on a triangulated height field (planar facets,
slope at most 20 deg), a 1 000-landmark submap, 15 Gauss-Newton iterations,
the reference's two-step pose.  The keyframe loop, the scene generator and
the host map manager are `sloam_gb300.trajectory`; this driver adds the
oracle leg, which only a comparison run (and the tests) may load.
"""
import argparse
import ctypes as C
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from sloam_gb300 import synth  # noqa: E402
from sloam_gb300 import trajectory as TJ  # noqa: E402


def oracle_keyframe_fn(L, s):
    """One keyframe through the oracle (same signature as
    `trajectory.gpu_keyframe_fn`'s closure)."""
    from sloam_gb300 import capi as A

    def kf(P, xyzi, lab, pose, mp):
        r = A.RunBuffers(P)
        mapc = A.cylinders_from_array(mp) if len(mp) else None
        st = L.oracle_keyframe(s, A.ptr(xyzi, C.c_float), len(xyzi), A.ptr(lab, C.c_uint8), None,
                               C.byref(A.SE3.from_qt(synth.quat_from_R(pose[0]), pose[1])), mapc,
                               len(mp), C.byref(r.s))
        r.refresh()
        q, t = r.s.T_Map_Curr.qt()
        n = r.s.models.n_cylinders
        return st, r.s.success, (synth.R_from_quat(q), t), r.m.cyl_array()[:n], r.matches[:n]
    return kf


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kf", type=int, default=200)
    ap.add_argument("--h", type=int, default=128)
    ap.add_argument("--w", type=int, default=2048)
    ap.add_argument("--trees", type=int, default=1000)
    ap.add_argument("--submap", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--oracle", type=int, default=1, help="also run the CPU restatement")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    import torch
    from sloam_gb300 import build, proposal
    build.build()
    from sloam_gb300.lib import Context, DeviceMapManager
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t0 = time.perf_counter()
    poses, odo, forest, terrain, scans = TJ.scene(a.seed, a.kf, a.h, a.w, a.trees, dev)
    gen_s = time.perf_counter() - t0
    res = {"config": {"keyframes": a.kf, "H": a.h, "W": a.w, "trees": a.trees,
                      "submap": a.submap, "gn_iters": 15, "seed": a.seed,
                      "scene_seconds": gen_s}}
    ests = {}
    for name, mode in (("gpu_plain", 1), ("gpu_learned", 2)):
        P = TJ.params(a.h, a.w, mode, submap=a.submap)
        ctx = Context(P)
        if mode == 2:
            ctx.set_proposal_weights(proposal.load_weights())
        est, dt = TJ.run(TJ.gpu_keyframe_fn(ctx), P, poses, odo, scans, a.submap)
        res[name] = dict(TJ.drift(poses, est), seconds=dt, keyframes_per_s=a.kf / dt)
        ests[name] = est
        ctx.close()
    # the plain path with the map manager on the GPU (sloam_keyframe_mapped)
    P = TJ.params(a.h, a.w, 1, submap=a.submap)
    ctx = Context(P)
    dm = DeviceMapManager(capacity=max(4 * a.trees, 4096), k=a.submap, recent=200)
    est, dt = TJ.run_mapped(ctx, dm, P, poses, odo, scans)
    dev_t = max(float(np.abs(np.asarray(e[1]) - np.asarray(h[1])).max())
                for e, h in zip(est, ests["gpu_plain"]))
    res["gpu_plain_device_map"] = dict(TJ.drift(poses, est), seconds=dt,
                                       keyframes_per_s=a.kf / dt,
                                       max_translation_diff_vs_host_map_m=dev_t,
                                       map_size=dm.size()[0])
    dm.close()
    ctx.close()
    if a.oracle:
        from oracle import loader
        loader.build()
        L = loader.lib()
        P = TJ.params(a.h, a.w, 1, submap=a.submap)
        s = L.oracle_create(C.byref(P))
        est, dt = TJ.run(oracle_keyframe_fn(L, s), P, poses, odo, scans, a.submap)
        L.oracle_destroy(s)
        res["cpu_reference_port"] = dict(TJ.drift(poses, est), seconds=dt,
                                         keyframes_per_s=a.kf / dt, threads=1)
        res["gpu_plain_vs_cpu_max_translation_diff_m"] = max(
            float(np.abs(np.asarray(e[1]) - np.asarray(h[1])).max())
            for e, h in zip(ests["gpu_plain"], est))
    odo_only = [poses[0]]
    for d in odo:
        odo_only.append(TJ._compose(odo_only[-1][0], odo_only[-1][1], *d))
    res["odometry_only"] = TJ.drift(poses, odo_only)
    line = json.dumps(res)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")


if __name__ == "__main__":
    main()
