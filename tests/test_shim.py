"""The C++ shim (the reference's host classes over the C ABI): the reference's
own C++ unit tests restated in tests/cpp/shim_test.cpp, fed the reference's
aux fixtures (from the golden npz) and a synthetic C2 keyframe pair."""
import os
import struct
import subprocess

import numpy as np
import pytest

from sloam_gb300 import capi as A
from sloam_gb300 import synth
from tests import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_test.cpp")


def _compile(out_dir):
    from sloam_gb300 import build
    build.build()
    exe = os.path.join(out_dir, "shim_test")
    lib_dir = os.path.dirname(build.SHIM_LIB)
    cmd = ["g++", "-O1", "-std=c++17", "-Wall", "-o", exe, SRC, "-L" + lib_dir,
           "-lsloam_shim", "-lsloam_gb300", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _write_landmarks(path, trees):
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(trees)))
        for tr in trees:
            f.write(struct.pack("<i", len(tr)))
            for v in tr:
                p = np.ascontiguousarray(v["points"][:, :3], np.float32)
                f.write(struct.pack("<id3fi", v["tree_id"], v["radius"], *map(float, v["xyz"]),
                                    len(p)))
                f.write(p.tobytes())


def _write_cloud(path, xyzi, h, w, labels=None):
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", h, w))
        f.write(np.ascontiguousarray(xyzi, np.float32).tobytes())
        if labels is not None:
            f.write(np.ascontiguousarray(labels, np.uint8).tobytes())


def _fixtures(d):
    for t in ("t0", "t1"):
        _write_landmarks(os.path.join(d, f"still_{t}.lm"), H.golden_landmarks("still", t))
        g = H.golden_ground(t)
        _write_cloud(os.path.join(d, f"still_{t}.ground"), g, 1, len(g))
    cloud, h, w = H.golden_tree_cloud("still", "t0")
    _write_cloud(os.path.join(d, "still_t0.tree"), cloud, h, w)
    # synthetic C2 pair; the staged-class comparison needs the vertex-line
    # cylinder mode (the staged landmarks carry no component clusters)
    cfg, forest, kfs = H.scene("C2", seed=0, n_kf=2)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=0)
    with open(os.path.join(d, "synth.params"), "wb") as f:
        f.write(bytes(P))
    with open(os.path.join(d, "synth.poses"), "wb") as f:
        for q, t in (kfs[0].pose_gt_qt(), kfs[1].pose_est_qt(), kfs[1].pose_gt_qt()):
            f.write(bytes(A.SE3.from_qt(q, t)))
    for k in range(2):
        _write_cloud(os.path.join(d, f"synth_kf{k}.scan"), kfs[k].xyzi, cfg.H, cfg.W,
                     kfs[k].labels)


def test_shim_builds_and_links(tmp_path):
    """The shim library and a program using it compile and link (no GPU)."""
    assert os.path.exists(_compile(str(tmp_path)))


@pytest.mark.gpu
def test_reference_cpp_tests_on_the_shim(tmp_path):
    exe = _compile(str(tmp_path))
    _fixtures(str(tmp_path))
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
