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
