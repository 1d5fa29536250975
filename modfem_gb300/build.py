"""Builds libmodfem_gb300.so in-tree with nvcc for sm_103a.

Translation units compile in parallel, then link into one shared library
next to this file.  Rebuilds only when a source is newer than the library.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libmodfem_gb300.so")
OBJDIR = os.path.join(HERE, "_build")
SOURCES = ["api.cu", "std_kernels.cu", "krylov.cu", "structure.cpp", "noalloc.cu", "dg_kernels.cu", "dg_faces.cu",
           "dg_krylov.cu", "serve.cu", "dg_tc.cu", "structure_gpu.cu", "io.cpp", "dg_batch.cu", "dg_tc_faces.cu", "dg_tet_faces.cu", "gmres_dev.cu", "dg_mixed_faces.cu"]
HEADERS = ["gbfem_internal.h", "prism_std.cuh", "prism_dw.cuh", "dword.cuh", "dg_face.cuh", "dg_spmv.cuh", "dg_volume.cuh", "tc_ptx.cuh", "dg_tables.h", os.path.join("..", "..", "include", "modfem_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for s in SOURCES + HEADERS + ["../build.py"]:
        if os.path.getmtime(os.path.join(CSRC, s)) > t:
            return True
    return False


def _compile(src):
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
           os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-x", "c++", "-c",
               os.path.join(CSRC, src), "-o", obj]
    subprocess.check_call(cmd)
    return obj


def build(force=False, verbose=True):
    if not force and not _stale():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
