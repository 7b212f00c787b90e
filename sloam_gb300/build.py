"""Builds libsloam_gb300.so in-tree with nvcc for sm_103a (no cmake), and
libsloam_shim.so (the reference's host classes over the C ABI) with g++.

Each translation unit compiles in parallel; host code is built with
-ffp-contract=off so the host-side boundary tables use the reference's
unfused float/double arithmetic.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "_build", "libsloam_gb300.so")
SHIM_SRC = os.path.join(HERE, "shim")
SHIM_LIB = os.path.join(HERE, "_build", "libsloam_shim.so")
UNITS = ["project.cu", "trellis.cu", "models.cu", "cylqueue.cu", "pose.cu", "context.cu",
         "noalloc.cu", "proposal.cu", "ingest.cu", "mapmgr.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                  "-Xptxas", "-O3"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)] + [
        os.path.join(HERE, "..", "include", "sloam_gb300.h")]


def build_shim(force=False):
    """libsloam_shim.so: sloam_gb300/shim/*.cpp linked against the C ABI."""
    deps = [os.path.join(SHIM_SRC, f) for f in os.listdir(SHIM_SRC)] + [LIB]
    if not force and os.path.exists(SHIM_LIB) and \
            os.path.getmtime(SHIM_LIB) >= max(os.path.getmtime(f) for f in deps):
        return SHIM_LIB
    srcs = [os.path.join(SHIM_SRC, f) for f in sorted(os.listdir(SHIM_SRC)) if f.endswith(".cpp")]
    tmp = SHIM_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-o", tmp, *srcs,
           "-L" + OUT, "-lsloam_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"shim build failed:\n{r.stderr}")
    os.replace(tmp, SHIM_LIB)
    return SHIM_LIB


def build(force=False, verbose=False, ptxas_v=False):
    lib = build_cuda(force, verbose, ptxas_v)
    build_shim(force)
    return lib


def build_cuda(force=False, verbose=False, ptxas_v=False):
    os.makedirs(OUT, exist_ok=True)
    newest = max(os.path.getmtime(f) for f in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    exe = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_v else []

    def one(u):
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        cmd = [exe, *NVFLAGS, *extra, "-c", os.path.join(SRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {u}:\n{r.stderr}")
        if verbose or ptxas_v:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB)
