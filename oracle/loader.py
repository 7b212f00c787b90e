"""TEST INFRASTRUCTURE ONLY: ctypes loader of the CPU oracle
(oracle/sloam_oracle.cpp).  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg; never by the sloam_gb300 package."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "sloam_oracle.cpp")

# -ffp-contract=off keeps float expressions unfused (the reference's x86-64
# build has no FMA), on both x86-64 and aarch64 hosts.
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "sloam_oracle.h")))):
        return LIB
    cmd = ["g++", *CXXFLAGS, SRC, "-o", LIB]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(LIB)
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from sloam_gb300 import capi as A
    vp = C.c_void_p
    L.oracle_project_mask.argtypes = [C.POINTER(A.Params), C.POINTER(C.c_float), C.c_int32,
                                      C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), C.c_int,
                                      C.POINTER(A.ScanOut)]
    L.oracle_trellis.argtypes = [C.POINTER(A.Params), C.POINTER(C.c_float), C.c_int32, C.c_int32,
                                 C.c_int, C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_int32),
                                 C.POINTER(A.Landmarks)]
    L.oracle_create.restype = vp
    L.oracle_create.argtypes = [C.POINTER(A.Params)]
    L.oracle_destroy.argtypes = [vp]
    L.oracle_set_params.argtypes = [vp, C.POINTER(A.Params)]
    L.oracle_reset.argtypes = [vp]
    L.oracle_compute_models.argtypes = [vp, C.POINTER(A.SE3), C.POINTER(C.c_float), C.c_int32,
                                        C.POINTER(A.Landmarks), C.POINTER(A.ModelsOut)]
    L.oracle_run.argtypes = [vp, C.POINTER(A.SE3), C.POINTER(C.c_float), C.c_int32,
                             C.POINTER(A.Landmarks), C.POINTER(A.Cylinder), C.c_int32,
                             C.POINTER(A.RunOut)]
    L.oracle_keyframe.argtypes = [vp, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_uint8),
                                  C.POINTER(C.c_uint8), C.POINTER(A.SE3), C.POINTER(A.Cylinder),
                                  C.c_int32, C.POINTER(A.RunOut)]
    L.oracle_plane.argtypes = [C.POINTER(A.Params), C.POINTER(C.c_float), C.c_int32,
                               C.POINTER(A.Plane), C.POINTER(C.c_float)]
    L.oracle_cylinder.argtypes = [C.POINTER(A.Params), C.POINTER(A.Landmarks), C.c_int32,
                                  C.POINTER(A.Plane), C.POINTER(A.Cylinder), C.POINTER(C.c_float),
                                  C.POINTER(C.c_int32)]
    L.oracle_cylinder_distance_model.restype = C.c_double
    L.oracle_cylinder_distance_model.argtypes = [C.POINTER(A.Cylinder), C.POINTER(A.Cylinder)]
    L.oracle_cylinder_distance_point.restype = C.c_double
    L.oracle_cylinder_distance_point.argtypes = [C.POINTER(A.Cylinder), C.POINTER(C.c_float)]
    L.oracle_cylinder_project.argtypes = [C.POINTER(A.Cylinder), C.POINTER(A.SE3)]
    L.oracle_plane_distance_point.restype = C.c_double
    L.oracle_plane_distance_point.argtypes = [C.POINTER(A.Plane), C.POINTER(C.c_float)]
    L.oracle_plane_project.argtypes = [C.POINTER(A.Plane), C.POINTER(A.SE3)]
    L.oracle_philox.argtypes = [C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.oracle_eigen_svd_u3.argtypes = [C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double)]
    _lib = L
    return L
