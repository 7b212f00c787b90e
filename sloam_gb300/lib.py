"""ctypes binding of libsloam_gb300.so (the CUDA C ABI of include/sloam_gb300.h).

There is no CPU fallback: importing the binding without the built library, or
creating a context without a CUDA device, raises.
"""
import ctypes as C
import os

from . import capi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsloam_gb300.so")

EXPORTS = [
    "sloam_params_default", "sloam_abi_sizes", "sloam_create", "sloam_destroy",
    "sloam_last_error", "sloam_reset", "sloam_set_params", "sloam_project_mask",
    "sloam_trellis", "sloam_compute_models", "sloam_fit_plane", "sloam_fit_cylinders",
    "sloam_run", "sloam_keyframe",
    "sloam_keyframes_device", "sloam_keyframes_host", "sloam_last_launch_count", "sloam_stream",
    "sloam_internal_tables", "sloam_set_proposal_weights", "sloam_pack_points",
    "sloam_mapmgr_create", "sloam_mapmgr_destroy", "sloam_mapmgr_size", "sloam_mapmgr_read",
    "sloam_mapmgr_load", "sloam_mapmgr_submap", "sloam_keyframe_mapped", "sloam_set_cc_iter_limit",
    "sloam_batch_scan_out", "sloam_frontend_time",
]

_lib = None


class SloamError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{A.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def load(path=LIB_PATH):
    """Loads the library (it must have been built: sloam_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m sloam_gb300.build`")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.sloam_params_default.argtypes = [C.POINTER(A.Params)]
    L.sloam_abi_sizes.argtypes = [C.POINTER(C.c_int32), C.c_int]
    L.sloam_abi_sizes.restype = C.c_int
    L.sloam_create.argtypes = [C.POINTER(A.Params), C.c_int, C.POINTER(C.c_int)]
    L.sloam_create.restype = vp
    L.sloam_destroy.argtypes = [vp]
    L.sloam_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.sloam_reset.argtypes = [vp]
    L.sloam_set_params.argtypes = [vp, C.POINTER(A.Params)]
    L.sloam_project_mask.argtypes = [vp, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_uint8),
                                     C.POINTER(C.c_uint8), C.POINTER(A.ScanOut)]
    L.sloam_trellis.argtypes = [vp, C.POINTER(C.c_float), C.c_int32, C.c_int32,
                                C.POINTER(C.c_uint32), C.POINTER(C.c_int32),
                                C.POINTER(A.Landmarks)]
    L.sloam_compute_models.argtypes = [vp, C.POINTER(A.SE3), C.POINTER(C.c_float), C.c_int32,
                                       C.POINTER(A.Landmarks), C.POINTER(A.ModelsOut)]
    L.sloam_fit_plane.argtypes = [vp, C.POINTER(C.c_float), C.c_int32, C.POINTER(A.Plane),
                                  C.POINTER(C.c_float)]
    L.sloam_fit_cylinders.argtypes = [vp, C.POINTER(A.Landmarks), C.POINTER(A.Plane), C.c_int32,
                                      C.POINTER(A.ModelsOut)]
    L.sloam_run.argtypes = [vp, C.POINTER(A.SE3), C.POINTER(C.c_float), C.c_int32,
                            C.POINTER(A.Landmarks), C.POINTER(A.Cylinder), C.c_int32,
                            C.POINTER(A.RunOut)]
    L.sloam_keyframe.argtypes = [vp, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_uint8),
                                 C.POINTER(C.c_uint8), C.POINTER(A.SE3), C.POINTER(A.Cylinder),
                                 C.c_int32, C.POINTER(A.RunOut)]
    L.sloam_keyframes_device.argtypes = [vp, vp, C.c_int32, C.c_int32, vp, C.POINTER(A.SE3),
                                         vp, C.c_int32, vp, vp, vp]
    L.sloam_keyframes_host.argtypes = [vp, vp, C.c_int32, C.c_int32, vp, C.POINTER(A.SE3),
                                       C.POINTER(A.Cylinder), C.c_int32, vp, vp, vp]
    L.sloam_project_mask_noalloc.argtypes = [C.POINTER(A.Params), vp, C.c_int32, vp, vp, vp, vp,
                                             vp, vp, vp, vp, vp]
    L.sloam_set_proposal_weights.argtypes = [vp, C.POINTER(C.c_float), C.c_int32]
    L.sloam_set_cc_iter_limit.argtypes = [vp, C.c_int32]
    L.sloam_pack_points.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_int32, vp, vp]
    L.sloam_mapmgr_create.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                      C.POINTER(vp)]
    L.sloam_mapmgr_destroy.argtypes = [vp]
    L.sloam_mapmgr_size.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32)]
    L.sloam_mapmgr_read.argtypes = [vp, C.POINTER(A.Cylinder), C.POINTER(C.c_int32), C.c_int32,
                                    C.POINTER(C.c_int32)]
    L.sloam_mapmgr_load.argtypes = [vp, C.POINTER(A.Cylinder), C.POINTER(C.c_int32), C.c_int32]
    L.sloam_mapmgr_submap.argtypes = [vp, C.c_double, C.c_double, C.POINTER(A.Cylinder),
                                      C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32)]
    L.sloam_keyframe_mapped.argtypes = [vp, vp, C.POINTER(C.c_float), C.c_int32,
                                        C.POINTER(C.c_uint8), C.POINTER(C.c_uint8),
                                        C.POINTER(A.SE3), C.POINTER(A.RunOut)]
    L.sloam_last_launch_count.argtypes = [vp]
    L.sloam_last_launch_count.restype = C.c_int64
    L.sloam_stream.argtypes = [vp]
    L.sloam_stream.restype = vp
    # profiling hooks (not in the public header)
    L.sloam_profile_stages.argtypes = [vp, C.POINTER(C.c_float), C.c_int]
    L.sloam_time_kernel.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.sloam_frontend_time.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32)]
    L.sloam_batch_scan_out.argtypes = [vp, C.c_int32, C.POINTER(A.ScanOut)]
    L.sloam_keyframe_stats.argtypes = [vp, C.POINTER(C.c_int32), C.c_int]
    _lib = L
    return L


class Context:
    """Owns one sloam_ctx (one device arena + one CUDA stream)."""

    def __init__(self, params=None, device=0):
        self.L = load()
        self.params = params if params is not None else A.default_params()
        st = C.c_int(0)
        self.h = self.L.sloam_create(C.byref(self.params), device, C.byref(st))
        if not self.h:
            raise SloamError(st.value, "sloam_create failed (is a CUDA device visible?)")

    def close(self):
        if getattr(self, "h", None):
            self.L.sloam_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def error(self):
        buf = C.create_string_buffer(512)
        self.L.sloam_last_error(self.h, buf, 512)
        return buf.value.decode()

    def check(self, st, ok=(A.SLOAM_OK,)):
        if st not in ok:
            raise SloamError(st, self.error())
        return st

    def set_proposal_weights(self, w):
        """Loads the learned-proposal weights (FP32, 75 399 values)."""
        import numpy as np
        w = np.ascontiguousarray(w, np.float32)
        self.check(self.L.sloam_set_proposal_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)),
                                                     w.size))

    def launches(self):
        return int(self.L.sloam_last_launch_count(self.h))

    def stream(self):
        return self.L.sloam_stream(self.h)


class DeviceMapManager:
    """The map manager on the GPU (sloam_mapmgr_*): map, hit counts, submap
    query and update in device memory."""

    def __init__(self, capacity=100000, k=100, recent=200, device=0):
        self.L = load()
        h = C.c_void_p()
        st = self.L.sloam_mapmgr_create(device, capacity, k, recent, C.byref(h))
        if st:
            raise SloamError(st, "sloam_mapmgr_create failed")
        self.h = h
        self.capacity = capacity

    def close(self):
        if getattr(self, "h", None):
            self.L.sloam_mapmgr_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def size(self):
        n, s, o = C.c_int32(), C.c_int32(), C.c_int32()
        st = self.L.sloam_mapmgr_size(self.h, C.byref(n), C.byref(s), C.byref(o))
        if st:
            raise SloamError(st)
        return n.value, s.value, o.value

    def read(self):
        """(models [n, 8] = root3, ray3, radius, id; hits [n])."""
        import numpy as np
        n = self.size()[0]
        arr = (A.Cylinder * max(1, n))()
        hits = np.zeros(max(1, n), np.int32)
        got = C.c_int32()
        st = self.L.sloam_mapmgr_read(self.h, arr, hits.ctypes.data_as(C.POINTER(C.c_int32)),
                                      n, C.byref(got))
        if st:
            raise SloamError(st)
        return A.cylinders_to_array(arr, n), hits[:n]

    def load(self, models, hits):
        import numpy as np
        n = len(models)
        arr = A.cylinders_from_array(np.asarray(models, np.float64).reshape(-1, 8))
        h = np.ascontiguousarray(hits, np.int32)
        st = self.L.sloam_mapmgr_load(self.h, arr, h.ctypes.data_as(C.POINTER(C.c_int32)), n)
        if st:
            raise SloamError(st)

    def submap(self, x, y, cap=4096):
        """(submap models [m, 8], their map indices [m])."""
        import numpy as np
        arr = (A.Cylinder * cap)()
        idx = np.zeros(cap, np.int32)
        n = C.c_int32()
        st = self.L.sloam_mapmgr_submap(self.h, x, y, arr, idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                        cap, C.byref(n))
        if st:
            raise SloamError(st)
        m = n.value
        return A.cylinders_to_array(arr, m), idx[:m]
