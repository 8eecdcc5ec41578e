"""The C-ABI library loads and exports every function include/rayspace3d.h declares
(no compute calls: these tests run without a GPU)."""
import os
import re
import subprocess

import pytest

from rayspace3d_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rayspace3d.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "sizeof")))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(build.LIB_PATH):
        build.build_lib()
    return _lib.load()


# Declared with C++ linkage, as the reference declares them (estimated_overlap.h:6-13,
# estimated_intersection.h:6-13); ctypes reaches them through their rs_ C forms.
CXX_LINKAGE = {"estimateOverlapSelectivity", "estimateIntersectionSelectivity"}


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ["rs_bvh_build", "rs_pim", "rs_pim_filtered", "rs_edge_join", "rs_containment",
              "rs_pairset_finalize", "rs_estimate_grid", "exclusive_scan_gpu", "merge_and_deduplicate_pairs_gpu",
              "compact_hash_table_pairs", "count_hits_gpu", "compact_hits_gpu", "estimateOverlapSelectivity",
              "estimateIntersectionSelectivity", "rs_pairset_set_edge_rule"]:
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "-C", "--defined-only", build.LIB_PATH], stdout=subprocess.PIPE, text=True,
                         check=True).stdout
    exported = set()
    for line in out.splitlines():
        parts = line.split(maxsplit=2)
        if len(parts) == 3:
            exported.add(parts[2].split("(")[0])
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"not exported: {missing}"
    for n in declared_functions():
        if n in CXX_LINKAGE:
            continue
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"
        getattr(lib, n)


REF_LINK_TU = r"""
#include "estimated_overlap.h"
#include "estimated_intersection.h"
#include "scan_utils.h"
#include "mesh_query_deduplication.h"
#include "result_compaction.h"
int main(int argc, char**) {
    if (argc > 99) {  // never taken: the calls only need to link (they would need a GPU)
        estimateOverlapSelectivity(nullptr, nullptr, 0, 1.0f);
        estimateIntersectionSelectivity(nullptr, nullptr, 0, 1.0f, 0.001f, 0.8f);
        exclusive_scan_gpu(nullptr, nullptr, 0);
        merge_and_deduplicate_pairs_gpu(nullptr, 0, nullptr, 0, nullptr);
        compact_hash_table_pairs(nullptr, 0, nullptr, 0);
        count_hits_gpu(nullptr, 0);
        compact_hits_gpu(nullptr, nullptr, 0, nullptr);
    }
    return 0;
}
"""


def test_reference_declarations_link(lib, tmp_path):
    """A translation unit written against the reference's own headers (estimated_overlap.h,
    estimated_intersection.h, scan_utils.h, mesh_query_deduplication.h, result_compaction.h)
    links against librs.so and loads."""
    from oracle import ref_build
    cuda_dir = os.path.join(ref_build.REF, "query", "src", "cuda")
    if not os.path.isdir(cuda_dir):
        pytest.skip("reference sources not present")
    src = tmp_path / "link_ref.cpp"
    src.write_text(REF_LINK_TU)
    exe = tmp_path / "link_ref"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "oracle", "ref", "stub"), "-I",
                    ref_build.cuda_include(), "-I", cuda_dir, "-I", os.path.join(ref_build.REF, "common", "include"),
                    str(src), "-o", str(exe), "-L", os.path.dirname(build.LIB_PATH), "-lrs",
                    "-Wl,-rpath," + os.path.dirname(build.LIB_PATH)], check=True)
    assert subprocess.run([str(exe)]).returncode == 0


def test_host_only_helpers(lib):
    assert lib.rs_version().decode().startswith("rayspace3d-gb300")
    assert lib.rs_status_string(3).decode() == "pair table full"
    # hash sizing rules (raytracer_overlap_estimated_main.cpp:316-325,
    # raytracer_intersection_estimated_main.cpp:466-477)
    assert lib.rs_hash_size_pow2(0) == 16777216
    assert lib.rs_hash_size_pow2(1) == 1024
    assert lib.rs_hash_size_pow2(600) == 2048
    assert lib.rs_hash_size_pow2(1 << 40) == 1 << 30
    assert lib.rs_hash_size_odd(0, 0.5) == 16777216
    assert lib.rs_hash_size_odd(100, 0.5) == 1025
    assert lib.rs_hash_size_odd(5000, 0.5) == 10001
    assert lib.rs_hash_size_odd(5000, 0.25) == 20001


def test_estimate_pairs_from_raw(lib):
    import ctypes
    m = (ctypes.c_float * 4)(1.0, 1.0, 1.0, 1.0)
    # alpha = (1+1)^3 / 2 = 4 -> 100 / 4
    assert lib.rs_estimate_pairs_from_raw(100.0, m, 2.0, 1) == 25
    assert lib.rs_estimate_pairs_from_raw(100.0, m, 2.0, 0) == 100
    assert lib.rs_estimate_pairs_from_raw(100.0, m, 1000.0, 1) == 100  # alpha clamps to 1
