"""Converts the reference's own test fixtures into compact arrays.

Reads (from a KumarRobotics/sloam checkout given on the command line):
  sloam/src/tests/aux/{still,moving}_tree_t{0,1}.pcd   organised 64x2048 tree clouds
  sloam/src/tests/aux/{still,moving}_landmarks_t{0,1}  Boost text archives of the
                                                        Trellis output for each cloud
  sloam/src/tests/aux/still_ground_t{0,1}.pcd          ground clouds (core_test.cpp)
and writes tests/golden/reference_aux.npz.  The tree clouds are stored sparse
(flat pixel index + x,y,z,intensity of the finite pixels); every value is the
float32 that pcl::io::loadPCDFile would parse from the text.

Archive layout (serialization.h:13-31, Boost text archive v17): a
vector<vector<TreeVertex>>; each collection is `count item_version`; each
TreeVertex is `treeId beam prevVertexSize radius isValid coords points` with
coords = x y z and points a collection of x y z; the first occurrence of every
class is preceded by a `0 0` class-info pair.

Usage: python tests/golden/make_golden.py <reference_root>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_pcd(path):
    with open(path) as f:
        header = {}
        while True:
            line = f.readline()
            k, *v = line.split()
            header[k] = v
            if k == "DATA":
                assert v[0] == "ascii"
                break
        w, h = int(header["WIDTH"][0]), int(header["HEIGHT"][0])
        data = np.loadtxt(f, dtype=np.float32).reshape(-1, 4)
    assert data.shape[0] == w * h
    return data, w, h


def read_landmarks(path):
    toks = open(path).read().split()
    assert toks[1] == "serialization::archive"
    pos = 3
    first = {"tree": True, "vtx": True, "pt": True, "pts": True}

    def take(n=1):
        nonlocal pos
        v = toks[pos:pos + n]
        pos += n
        return v

    def class_info(kind):
        if first[kind]:
            a, b = take(2)
            assert (a, b) == ("0", "0"), (kind, a, b, pos)
            first[kind] = False

    a, b = take(2)  # outer vector class info
    ntrees, _ = int(take()[0]), take()
    trees = []
    for _t in range(ntrees):
        class_info("tree")
        nv, _ = int(take()[0]), take()
        verts = []
        for _v in range(nv):
            class_info("vtx")
            tid, beam, prev = (int(x) for x in take(3))
            radius = float(take()[0])
            valid = int(take()[0])
            class_info("pt")
            xyz = np.array(take(3), np.float32)
            class_info("pts")
            npts, _ = int(take()[0]), take()
            pts = np.array(take(3 * npts), np.float32).reshape(npts, 3)
            verts.append((tid, beam, prev, radius, valid, xyz, pts))
        trees.append(verts)
    assert pos == len(toks), (pos, len(toks))
    return trees


def main(root):
    aux = os.path.join(root, "sloam", "src", "tests", "aux")
    out = {}
    for seq in ("still", "moving"):
        for t in ("t0", "t1"):
            cloud, w, h = read_pcd(os.path.join(aux, f"{seq}_tree_{t}.pcd"))
            fin = np.isfinite(cloud[:, 0])
            idx = np.nonzero(fin)[0].astype(np.int32)
            out[f"{seq}_{t}_tree_idx"] = idx
            out[f"{seq}_{t}_tree_xyzi"] = cloud[idx]
            out[f"{seq}_{t}_tree_hw"] = np.array([h, w], np.int32)
            trees = read_landmarks(os.path.join(aux, f"{seq}_landmarks_{t}"))
            vt, vx, vr, pb, pts, lb = [], [], [], [0], [], [0]
            for tr in trees:
                for (tid, beam, prev, radius, valid, xyz, p) in tr:
                    vt.append(tid)
                    vx.append(xyz)
                    vr.append(radius)
                    pts.append(p)
                    pb.append(pb[-1] + len(p))
                lb.append(lb[-1] + len(tr))
            out[f"{seq}_{t}_lm_vertex_tree"] = np.array(vt, np.int32)
            out[f"{seq}_{t}_lm_vertex_xyz"] = np.array(vx, np.float32)
            out[f"{seq}_{t}_lm_vertex_radius"] = np.array(vr, np.float64)
            out[f"{seq}_{t}_lm_point_begin"] = np.array(pb, np.int32)
            out[f"{seq}_{t}_lm_points"] = np.concatenate(pts).astype(np.float32)
            out[f"{seq}_{t}_lm_vertex_begin"] = np.array(lb, np.int32)
    for t in ("t0", "t1"):
        g, _, _ = read_pcd(os.path.join(aux, f"still_ground_{t}.pcd"))
        out[f"still_{t}_ground"] = g
    dst = os.path.join(HERE, "reference_aux.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference_root>")
    main(sys.argv[1])
