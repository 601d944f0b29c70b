"""Builds kfr_gb300/lib/libkfr_capi.so: the CUDA kernels for sm_103a and the C ABI, in parallel.

    python -m kfr_gb300.build [--force] [--jobs N]

Objects go to kfr_gb300/_build/ and are rebuilt when any source or header is newer.  The CUDA runtime is
linked statically, so the library depends only on the NVIDIA driver.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libkfr_capi.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = [
    "kernels_f32.cu", "kernels_f64.cu", "kernels_ct_a.cu", "kernels_ct_b.cu", "kernels_ct_c.cu", "elementwise.cu",
    "conv.cu", "convolve.cu", "adjoint.cu", "uneven.cu", "tensor.cu", "static_scratch.cu", "rader_pfa.cu",
]
CPP_SOURCES = ["plan.cpp", "md.cpp", "capi.cpp", "launch_cache.cpp"]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    common = ["-std=c++17", "-O3", "-I", CSRC, "-I", INCLUDE]
    cmds = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            cmds.append([NVCC] + common + ARCH + ["-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-Xptxas", "-v",
                                                  "-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            cmds.append(["g++"] + common + ["-fPIC", "-Wall", "-Wno-unused-function", "-fvisibility=hidden",
                                            "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj])
    if cmds:
        jobs = jobs or min(len(cmds), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for out in ex.map(_compile, cmds):
                if verbose and out:
                    print(out)
    if cmds or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        # export the C ABI only
        vscript = os.path.join(BUILD, "exports.map")
        with open(vscript, "w") as f:
            f.write("{ global: kfr_*; local: *; };\n")
        link = [NVCC, "-shared", "-cudart", "static"] + ARCH + ["-o", tmp] + objs + [
            "-lpthread", "-ldl", "-lrt", "-Xlinker", "--exclude-libs,ALL", "-Xlinker", "--version-script=" + vscript]
        _compile(link)
        shutil.move(tmp, LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.force, a.jobs, a.verbose))


if __name__ == "__main__":
    sys.exit(main())
