"""Build recipe for libtfgpu.so (the CUDA path) -- nvcc for sm_103a only.

The library is built in-tree into ``tissuefolding_paperversion_gb300/_lib``;
object files go to ``_build``.  Translation units compile in parallel.
``build(checked=True)`` builds libtfgpu_checked.so (-DTF_CHECKED: every
checked index is tested before its access; a failed test is reported as
TF_CUDA_ERROR instead of touching memory out of bounds) into ``_build_checked``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libtfgpu.so")
LIB_CHECKED = os.path.join(LIBDIR, "libtfgpu_checked.so")
SOURCES = ["tf_api.cu", "tf_element.cu", "tf_assembly.cu", "tf_krylov.cu", "tf_static_solve.cu", "tf_adjoint.cu", "tf_amg.cu",
           "tf_packing.cu", "tf_growth.cu", "tf_probe.cu", "tf_meshio.cpp"]
HEADERS = ["tf_internal.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libtfgpu")
    return p


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    obj_dir = OBJ + "_checked" if checked else OBJ
    lib = LIB_CHECKED if checked else LIB
    flags = FLAGS + (["-DTF_CHECKED"] if checked else [])
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "tf_gpu.h")]
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(obj_dir, os.path.splitext(s)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs]):
            jobs.append([nvcc(), *ARCH, *flags, "-c", src, "-o", obj])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(lib, objs):
        run([nvcc(), *ARCH, "-shared", "-o", lib, *objs])
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
