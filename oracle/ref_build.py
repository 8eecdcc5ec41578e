"""Recipe: compile pieces of the reference's own host code into oracle/_ref/ref_driver.

Test infrastructure.  Compiles, where they lie under /root/reference, the reference's
EdgePreprocessor.cpp, timer.cpp, PointIO.cpp and BoundingBox.cpp (plus the header-only
BinaryIO.h) together with oracle/ref/ref_driver.cpp, a host-memory shim for
cudaMallocHost/cudaFreeHost (oracle/ref/pinned_shim.cpp) and a one-line stand-in for the
OptiX header.  preprocess_dataset.cpp is compiled with its main() renamed, for
generateGridStats only; its dataset loaders are replaced by never-called stand-ins
(oracle/ref/loader_stub.cpp).  The OptiX device programs and the CGAL/tinyobjloader preprocess loaders
cannot be built here and are not part of this recipe.  Outputs go to oracle/_ref/ only.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = "/root/reference"
OUT = os.path.join(HERE, "_ref")
DRIVER = os.path.join(OUT, "ref_driver")

SOURCES = ["preprocess/src/EdgePreprocessor.cpp", "query/src/timer.cpp", "query/src/runtime/PointIO.cpp",
           "query/src/geometry/BoundingBox.cpp"]
RENAMED_MAIN = "preprocess/src/preprocess_dataset.cpp"  # compiled alone, main() renamed
INCLUDES = ["query/src", "common/include", "preprocess/src", "query/src/runtime", "query/src/geometry"]  # query timer.h first


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
        return DRIVER
    base = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", os.path.join(HERE, "ref", "stub"),
            "-I", cuda_include()]
    for inc in INCLUDES:
        base += ["-I", os.path.join(REF, inc)]
    obj = os.path.join(OUT, "preprocess_dataset.o")
    subprocess.run(base + ["-Dmain=ref_preprocess_main", "-c", renamed, "-o", obj], check=True)
    subprocess.run(base + srcs + [obj, "-o", DRIVER], check=True)
    return DRIVER


if __name__ == "__main__":
    print(build(force=True))
