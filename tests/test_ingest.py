"""Input ingestion: PointCloud2-layout points packed into float4 XYZI."""
import numpy as np
import pytest

from sloam_gb300 import capi as A

pytestmark = pytest.mark.gpu


def _cloud(n, rng):
    # an Ouster-like layout: 48 bytes per point; x, y, z, intensity float32
    # at 0, 4, 8, 16; reflectivity uint16 at 24; ring uint8 at 26
    rec = np.zeros(n, dtype=[("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("pad", "<f4"),
                             ("intensity", "<f4"), ("t", "<u4"), ("refl", "<u2"), ("ring", "u1"),
                             ("pad2", "u1"), ("rest", "u1", 20)])
    assert rec.dtype.itemsize == 48
    for k in ("x", "y", "z", "intensity"):
        rec[k] = rng.normal(size=n).astype(np.float32) * 10
    rec["refl"] = rng.integers(0, 65535, n)
    rec["ring"] = rng.integers(0, 128, n)
    rec["x"][::97] = np.nan
    return rec


@pytest.mark.parametrize("field,itype", [("intensity", 1), ("refl", 2), ("ring", 3), (None, 0)])
def test_pack_points_matches_numpy(field, itype):
    import torch
    from sloam_gb300.lib import load
    L = load()
    rng = np.random.default_rng(0)
    n = 100003
    rec = _cloud(n, rng)
    off = {"intensity": 16, "refl": 24, "ring": 26, None: 0}[field]
    src = torch.from_numpy(rec.view(np.uint8).copy()).cuda()
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    st = L.sloam_pack_points(src.data_ptr(), n, 48, 0, 4, 8, off, itype, out.data_ptr(), None)
    assert st == A.SLOAM_OK
    got = out.cpu().numpy()
    exp = np.zeros((n, 4), np.float32)
    exp[:, 0], exp[:, 1], exp[:, 2] = rec["x"], rec["y"], rec["z"]
    if field is not None:
        exp[:, 3] = rec[field].astype(np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_pack_points_unaligned_layout():
    import torch
    from sloam_gb300.lib import load
    L = load()
    n = 5001
    rng = np.random.default_rng(1)
    xyz = rng.normal(size=(n, 3)).astype(np.float32)
    raw = np.zeros((n, 15), np.uint8)  # 15-byte points, fields at 1, 5, 9, intensity u8 at 13
    for k in range(3):
        raw[:, 1 + 4 * k:5 + 4 * k] = xyz[:, k:k + 1].view(np.uint8)
    raw[:, 13] = rng.integers(0, 255, n)
    src = torch.from_numpy(raw.reshape(-1).copy()).cuda()
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    assert L.sloam_pack_points(src.data_ptr(), n, 15, 1, 5, 9, 13, 3, out.data_ptr(), None) == 0
    got = out.cpu().numpy()
    np.testing.assert_array_equal(got[:, :3], xyz)
    np.testing.assert_array_equal(got[:, 3], raw[:, 13].astype(np.float32))


def test_pack_points_rejects_fields_outside_the_point():
    from sloam_gb300.lib import load
    L = load()
    assert L.sloam_pack_points(None, 0, 16, 0, 4, 8, 12, 1, None, None) == A.SLOAM_OK
    assert L.sloam_pack_points(1, 10, 16, 0, 4, 14, 12, 1, 1, None) == A.SLOAM_ERR_ARG
