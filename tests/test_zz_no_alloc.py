"""sloam_project_mask_noalloc: projection + masking without any device
allocation, for callers that cannot call cudaMalloc (plugins inside a process
whose allocator owns the GPU, real-time loops that forbid allocation after
start-up).  Its scratch is a fixed file-scope device array shared by every
call; this file is collected last so that a failure here comes after every
other test has run."""
import ctypes as C

import numpy as np
import pytest

from sloam_gb300 import capi as A
from sloam_gb300 import synth
from tests import helpers as H


def _lib():
    from sloam_gb300 import build, lib
    build.build()
    return lib.load()


def test_noalloc_rejects_oversized_scans():
    L = _lib()
    P = A.default_params(img_w=4096, img_h=64)  # 262144 points > 131072
    n = P.img_w * P.img_h
    dummy = C.c_void_p(16)
    st = L.sloam_project_mask_noalloc(C.byref(P), dummy, n, dummy, None, None, None, None,
                                      dummy, dummy, dummy, None)
    assert st == A.SLOAM_ERR_CAPACITY


@pytest.mark.gpu
def test_noalloc_matches_existing_entry_point_twice():
    import torch
    from sloam_gb300.lib import Context
    L = _lib()
    cfg, forest, kfs = H.scene("C2", seed=0, n_kf=2)
    P = synth.preset_params(cfg, do_destagger=1)
    ctx = Context(P)
    n = P.img_w * P.img_h
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for kf in kfs:  # two calls in a row, different scans
        ref = H.gpu_project(ctx, kf.xyzi, labels=kf.labels)
        x = torch.from_numpy(kf.xyzi).to(dev)
        lab = torch.from_numpy(kf.labels).to(dev)
        pix = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rng = torch.zeros(n, dtype=torch.float32, device=dev)
        msk = torch.zeros(n, dtype=torch.uint8, device=dev)
        gidx = torch.full((n,), -1, dtype=torch.int32, device=dev)
        ng = torch.zeros(1, dtype=torch.int32, device=dev)
        tree = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        st = L.sloam_project_mask_noalloc(C.byref(P), x.data_ptr(), n, lab.data_ptr(), None,
                                          pix.data_ptr(), rng.data_ptr(), msk.data_ptr(),
                                          gidx.data_ptr(), ng.data_ptr(), tree.data_ptr(),
                                          C.c_void_p(stream.cuda_stream))
        assert st == A.SLOAM_OK
        stream.synchronize()
        k = int(ng.item())
        assert k == ref["n_ground"]
        np.testing.assert_array_equal(pix.cpu().numpy(), ref["py"] * P.img_w + ref["px"])
        np.testing.assert_array_equal(rng.cpu().numpy().view(np.uint32),
                                      ref["range_image"].view(np.uint32))
        np.testing.assert_array_equal(msk.cpu().numpy(), ref["mask_out"])
        np.testing.assert_array_equal(gidx.cpu().numpy()[:k], ref["ground_idx"][:k])
        np.testing.assert_array_equal(tree.cpu().numpy().view(np.uint32),
                                      ref["tree_cloud"].view(np.uint32))
    ctx.close()


@pytest.mark.gpu
def test_noalloc_mask_image_and_optional_outputs():
    """The network-style input (a per-pixel mask image instead of point
    labels) against sloam_project_mask with the same mask, and a call that
    skips every optional output (pixel indices, range image, mask out):
    the ground list, its count and the tree cloud are unchanged."""
    import torch
    from sloam_gb300.lib import Context
    L = _lib()
    cfg, forest, kfs = H.scene("C2", seed=0, n_kf=2)
    P = synth.preset_params(cfg, do_destagger=1)
    ctx = Context(P)
    n = P.img_w * P.img_h
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    kf = kfs[1]
    mask = H.gpu_project(ctx, kf.xyzi, labels=kf.labels)["mask_out"].copy()
    ref = H.gpu_project(ctx, kf.xyzi, mask=mask)
    x = torch.from_numpy(kf.xyzi).to(dev)
    m = torch.from_numpy(mask).to(dev)
    for optional in (True, False):
        pix = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rng = torch.zeros(n, dtype=torch.float32, device=dev)
        msk = torch.zeros(n, dtype=torch.uint8, device=dev)
        gidx = torch.full((n,), -1, dtype=torch.int32, device=dev)
        ng = torch.zeros(1, dtype=torch.int32, device=dev)
        tree = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        st = L.sloam_project_mask_noalloc(
            C.byref(P), x.data_ptr(), n, None, m.data_ptr(),
            pix.data_ptr() if optional else None, rng.data_ptr() if optional else None,
            msk.data_ptr() if optional else None, gidx.data_ptr(), ng.data_ptr(),
            tree.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert st == A.SLOAM_OK
        stream.synchronize()
        k = int(ng.item())
        assert k == ref["n_ground"]
        np.testing.assert_array_equal(gidx.cpu().numpy()[:k], ref["ground_idx"][:k])
        np.testing.assert_array_equal(tree.cpu().numpy().view(np.uint32),
                                      ref["tree_cloud"].view(np.uint32))
        if optional:
            np.testing.assert_array_equal(pix.cpu().numpy(), ref["py"] * P.img_w + ref["px"])
            np.testing.assert_array_equal(rng.cpu().numpy().view(np.uint32),
                                          ref["range_image"].view(np.uint32))
            np.testing.assert_array_equal(msk.cpu().numpy(), ref["mask_out"])
        else:
            assert (pix == -1).all() and (rng == 0).all() and (msk == 0).all()
    ctx.close()
