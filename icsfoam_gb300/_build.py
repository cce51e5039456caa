"""In-tree build of the native libraries.

* libicshost.so - host C++ mesh-ordering utilities (g++).
* libicsgpu.so  - the CUDA hot path and its C ABI (nvcc, sm_103a only).

Translation units compile in parallel into ``_build/``; the shared objects
land next to this file so the package loads them in place.
"""

from __future__ import annotations

import glob
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
HOST_LIB = os.path.join(PKG, "libicshost.so")
GPU_LIB = os.path.join(PKG, "libicsgpu.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC,
           "--expt-relaxed-constexpr"]


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _stale(target, deps):
    return not os.path.exists(target) or os.path.getmtime(target) < _newest(deps)


def build_host(force: bool = False) -> str:
    src = os.path.join(CSRC, "host_mesh.cpp")
    if force or _stale(HOST_LIB, [src]):
        tmp = HOST_LIB + ".tmp"
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", tmp, src])
        os.replace(tmp, HOST_LIB)
    return HOST_LIB


def cuda_sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def build_gpu(force: bool = False, extra_flags=None) -> str:
    srcs = cuda_sources()
    hdrs = glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(INC, "icsfoam_gb300.h")]
    if not force and not _stale(GPU_LIB, srcs + hdrs):
        return GPU_LIB
    os.makedirs(BUILD, exist_ok=True)
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [NVCC] + ARCH + NVFLAGS + (extra_flags or []) + ["-c", s, "-o", o]
            procs.append((subprocess.Popen(cmd), s))
    failed = [s for p, s in procs if p.wait() != 0]
    if failed:
        raise RuntimeError("nvcc failed on: " + ", ".join(failed))
    tmp = GPU_LIB + ".tmp"
    subprocess.check_call([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lpthread"])
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


def build_all(force: bool = False):
    build_host(force)
    build_gpu(force)
