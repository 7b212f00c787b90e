"""The C ABI library without a GPU: it builds, loads, exports every symbol of
include/sloam_gb300.h, its struct layouts match the bindings, its defaults
match the reference configuration, and it refuses to run without a device."""
import ctypes as C
import os
import re

import pytest

from sloam_gb300 import capi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    from sloam_gb300 import build, lib
    build.build()
    return lib.load()


def header_functions():
    src = open(os.path.join(ROOT, "include", "sloam_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sloam_[a-z_]+)\s*\(", src)))


def test_exports_every_header_symbol(L):
    names = header_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(L, n), n


def test_struct_sizes_match_bindings(L):
    out = (C.c_int32 * 16)()
    k = L.sloam_abi_sizes(out, 16)
    py = [C.sizeof(A.Params), C.sizeof(A.SE3), C.sizeof(A.Landmarks), C.sizeof(A.Cylinder),
          C.sizeof(A.Plane), C.sizeof(A.ScanOut), C.sizeof(A.ModelsOut), C.sizeof(A.RunOut)]
    assert list(out[:k]) == py


def test_defaults_match_reference_yaml(L):
    p = A.Params()
    L.sloam_params_default(C.byref(p))
    q = A.default_params()
    assert p.as_dict() == q.as_dict()


def test_no_device_fails_loudly(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    st = C.c_int(0)
    p = A.default_params()
    h = L.sloam_create(C.byref(p), 0, C.byref(st))
    assert not h
    assert st.value == A.SLOAM_ERR_NO_DEVICE


def test_bad_params_rejected(L):
    st = C.c_int(0)
    p = A.default_params(img_w=0)
    assert not L.sloam_create(C.byref(p), 0, C.byref(st))
    assert st.value == A.SLOAM_ERR_ARG


def test_boundary_tables_reproduce_oracle_pixels_and_bins(L):
    """The host-built float boundary tables (column of a yaw, theta / radius
    bins of a ground point) give exactly the oracle's integers."""
    import numpy as np
    from tests import helpers as H
    P = A.default_params(img_w=2048, img_h=64)
    tab = np.zeros(P.img_w + 1, np.float32)
    tb = np.zeros(P.ground_theta_bins + 1, np.float32)
    rb = np.zeros(P.ground_radii_bins + 1, np.float32)
    lohi = np.zeros(2, np.float32)
    ptab = np.zeros(P.img_h + 1, np.float32)
    L.sloam_internal_tables(C.byref(P), A.ptr(tab, C.c_float), A.ptr(tb, C.c_float),
                            A.ptr(rb, C.c_float), A.ptr(lohi, C.c_float), A.ptr(ptab, C.c_float))
    assert np.all(np.diff(tab[1:-1]) > 0)
    rng = np.random.default_rng(5)
    n = P.img_w * P.img_h
    v = rng.normal(size=(n, 3)).astype(np.float32)
    xyzi = np.zeros((n, 4), np.float32)
    xyzi[:, :3] = v * rng.uniform(0.5, 40, (n, 1)).astype(np.float32)
    o = H.oracle_project(P, xyzi, labels=np.zeros(n, np.uint8))
    yaw = -np.arctan2(xyzi[:, 1].astype(np.float64), xyzi[:, 0].astype(np.float64)).astype(np.float32)
    px = np.searchsorted(tab[1:P.img_w], yaw, side="right")
    np.testing.assert_array_equal(px, o["px"])
    # rows: from the table on q = the float z / range (the pitch is the
    # float asin of q; |q| > 1 has a NaN pitch: row H - 1)
    x, y, z = xyzi[:, 0], xyzi[:, 1], xyzi[:, 2]
    rng3 = np.sqrt((x * x + y * y) + z * z)
    q = (z / rng3).astype(np.float32)
    assert np.all(np.diff(ptab[1:-1]) >= 0)
    py = P.img_h - 1 - np.searchsorted(ptab[1:P.img_h], q, side="right")
    py = np.where(np.abs(q) <= 1, py, P.img_h - 1)
    np.testing.assert_array_equal(py, o["py"])
    # boundary q values themselves, and their float neighbours, against the
    # reference's row formula through the correctly rounded asin
    qs = np.concatenate([ptab[1:P.img_h][np.isfinite(ptab[1:P.img_h])]])
    qs = np.concatenate([qs, np.nextafter(qs, -np.inf), np.nextafter(qs, np.inf)]).astype(np.float32)
    fd = np.float32(np.radians(22.5)); fov = np.float32(fd + fd)
    pitch = np.arcsin(qs.astype(np.float64)).astype(np.float32)
    t = ((pitch + fd) / fov).astype(np.float32)
    yy = np.floor(((np.float32(1) - t) * np.float32(P.img_h)).astype(np.float32))
    row = np.clip(yy, 0, P.img_h - 1).astype(int)
    py2 = P.img_h - 1 - np.searchsorted(ptab[1:P.img_h], qs, side="right")
    np.testing.assert_array_equal(py2, row)
    # ground bins: theta from the float atan2, radius window in double
    x, y = xyzi[:, 0], xyzi[:, 1]
    r = np.sqrt(x * x + y * y).astype(np.float32)
    inwin = (r.astype(np.float64) < P.max_ground_lidar_dist) & (r.astype(np.float64) > P.min_ground_lidar_dist)
    assert np.array_equal(inwin, (r >= lohi[0]) & (r <= lohi[1]))
    th = np.arctan2(y.astype(np.float64), x.astype(np.float64)).astype(np.float32)
    tref = np.clip(np.floor((3.14159265 + th.astype(np.float64)) / (2 * 3.14159265 / P.ground_theta_bins)),
                   0, P.ground_theta_bins - 1).astype(int)
    ttab = np.searchsorted(tb[1:P.ground_theta_bins], th, side="right")
    np.testing.assert_array_equal(ttab, tref)
    rref = np.clip(np.floor(r.astype(np.float64) / (P.max_ground_lidar_dist / P.ground_radii_bins)),
                   0, P.ground_radii_bins - 1).astype(int)
    rtab = np.searchsorted(rb[1:P.ground_radii_bins], r, side="right")
    np.testing.assert_array_equal(rtab[inwin], rref[inwin])
