"""Recipe: compile pieces of the reference's own host code into oracle/_ref/ref_driver.

Test infrastructure.  Compiles, where they lie under the reference checkout ($RS_REFERENCE_DIR,
default /root/reference), the reference's
EdgePreprocessor.cpp, timer.cpp, PointIO.cpp and BoundingBox.cpp (plus the header-only
BinaryIO.h) together with oracle/ref/ref_driver.cpp, a host-memory shim for
cudaMallocHost/cudaFreeHost (oracle/ref/pinned_shim.cpp) and a one-line stand-in for the
OptiX header.  preprocess_dataset.cpp is compiled with its main() renamed, for
generateGridStats only; its dataset loaders are replaced by never-called stand-ins
(oracle/ref/loader_stub.cpp).  The OptiX device programs and the CGAL/tinyobjloader preprocess loaders
cannot be built here and are not part of this recipe.  Outputs go to oracle/_ref/ only.

The reference's plain CUDA helpers (estimated_overlap.cu, estimated_intersection.cu,
mesh_query_deduplication.cu, result_compaction.cu) are compiled unmodified, device code
only, into one cubin each (build_cuda): oracle/ref_cuda.py loads them through the CUDA
driver API so that GPU tests can run the reference's own kernels beside the engine's.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("RS_REFERENCE_DIR", "/root/reference")  # where the reference sources lie
OUT = os.path.join(HERE, "_ref")
DRIVER = os.path.join(OUT, "ref_driver")

SOURCES = ["preprocess/src/EdgePreprocessor.cpp", "query/src/timer.cpp", "query/src/runtime/PointIO.cpp",
           "query/src/geometry/BoundingBox.cpp"]
RENAMED_MAIN = "preprocess/src/preprocess_dataset.cpp"  # compiled alone, main() renamed
INCLUDES = ["query/src", "common/include", "preprocess/src", "query/src/runtime", "query/src/geometry"]  # query timer.h first


CUDA_SOURCES = ["estimated_overlap", "estimated_intersection", "mesh_query_deduplication", "result_compaction"]


def cubin_path(name: str) -> str:
    return os.path.join(OUT, name + ".cubin")


def build_cuda(force: bool = False) -> list:
    """The reference's CUDA helper files, unmodified, into oracle/_ref/<name>.cubin (sm_103a)."""
    if not os.path.isdir(REF):
        raise RuntimeError("reference sources are not present on this machine")
    os.makedirs(OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = []
    for name in CUDA_SOURCES:
        src = os.path.join(REF, "query", "src", "cuda", name + ".cu")
        dst = cubin_path(name)
        out.append(dst)
        if not force and os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
            continue
        subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-I", os.path.join(HERE, "ref", "stub"), "-I", os.path.join(REF, "common", "include"),
                        "-I", os.path.join(REF, "query", "src", "cuda"), "-I", os.path.join(REF, "query", "src"),
                        "-o", dst, src], check=True)
    return out


def cuda_include() -> str:
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nv))), "include")


def available() -> bool:
    """True where the reference sources this recipe compiles are present."""
    return os.path.isdir(REF)


def build(force: bool = False) -> str:
    if not os.path.isdir(REF):
        raise RuntimeError("reference sources are not present on this machine")
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(REF, s) for s in SOURCES] + [os.path.join(HERE, "ref", "ref_driver.cpp"),
                                                      os.path.join(HERE, "ref", "pinned_shim.cpp"),
                                                      os.path.join(HERE, "ref", "loader_stub.cpp")]
    renamed = os.path.join(REF, RENAMED_MAIN)
    if not force and os.path.exists(DRIVER) and all(os.path.getmtime(DRIVER) >= os.path.getmtime(s)
                                                    for s in srcs + [renamed]):
        build_cuda()
        return DRIVER
    base = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", os.path.join(HERE, "ref", "stub"),
            "-I", cuda_include()]
    for inc in INCLUDES:
        base += ["-I", os.path.join(REF, inc)]
    obj = os.path.join(OUT, "preprocess_dataset.o")
    subprocess.run(base + ["-Dmain=ref_preprocess_main", "-c", renamed, "-o", obj], check=True)
    subprocess.run(base + srcs + [obj, "-o", DRIVER], check=True)
    build_cuda(force)
    return DRIVER


if __name__ == "__main__":
    print(build(force=True))
