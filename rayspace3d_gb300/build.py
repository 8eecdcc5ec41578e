"""Compile the engine for sm_103a, in tree.

Products (git-ignored, rebuilt on every machine):
  rayspace3d_gb300/lib/librs.so          -- CUDA engine behind include/rayspace3d.h
  rayspace3d_gb300/bin/raytracer*        -- drop-in executables of the reference CLI
Every translation unit is compiled in parallel; cudart is linked statically so
the library loads next to any PyTorch build.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
from typing import List

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
LIB_PATH = os.path.join(LIB, "librs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
HOST_FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]

CLI_APPS = ["raytracer", "raytracer_filter_refine", "raytracer_mesh_overlap", "raytracer_overlap_estimated",
            "raytracer_overlap_direct_estimation", "raytracer_intersection_estimated", "raytracer_containment",
            "preprocess_dataset"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd: List[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")


def _stale(target: str, deps: List[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_lib(jobs: int = 8) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                     glob.glob(os.path.join(ROOT, "include", "*.h")))
    objs = []
    cmds = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmds.append([nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    if cmds or _stale(LIB_PATH, objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB_PATH] + objs)
    return LIB_PATH


def build_cli(jobs: int = 8) -> List[str]:
    """Drop-in executables (C++ host code over librs.so)."""
    if not os.path.isdir(HOST):
        return []
    srcs_common = sorted(glob.glob(os.path.join(HOST, "common", "*.cpp")))
    os.makedirs(BIN, exist_ok=True)
    os.makedirs(os.path.join(BUILD, "host"), exist_ok=True)
    inc = ["-I", os.path.join(cuda_home(), "include"), "-I", HOST]
    headers = sorted(glob.glob(os.path.join(HOST, "**", "*.h"), recursive=True)) + [
        os.path.join(ROOT, "include", "rayspace3d.h"), os.path.join(HOST, "apps", "raytracer_overlap_estimated.cpp")]
    objs = []
    cmds = []
    for src in srcs_common:
        obj = os.path.join(BUILD, "host", os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmds.append(["g++"] + HOST_FLAGS + inc + ["-fPIC", "-c", src, "-o", obj])
    app_objs = {}
    for app in CLI_APPS:
        src = os.path.join(HOST, "apps", app + ".cpp")
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, "host", app + ".o")
        app_objs[app] = obj
        if _stale(obj, [src] + headers):
            cmds.append(["g++"] + HOST_FLAGS + inc + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    libdir = os.path.join(cuda_home(), "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(cuda_home(), "lib")
    outs = []
    link_cmds = []
    for app, obj in app_objs.items():
        exe = os.path.join(BIN, app)
        outs.append(exe)
        if _stale(exe, [obj] + objs + [LIB_PATH]):
            link_cmds.append(["g++", "-o", exe, obj] + objs +
                             ["-L", LIB, "-lrs", "-Wl,-rpath,$ORIGIN/../lib", "-L", libdir, "-lcudart", "-lpthread",
                              "-Wl,-rpath," + libdir])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, link_cmds))
    return outs


def build_all(jobs: int = 8) -> None:
    build_lib(jobs)
    build_cli(jobs)


if __name__ == "__main__":
    build_all()
    print(LIB_PATH)
    sys.exit(0)
