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


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ["rs_bvh_build", "rs_pim", "rs_pim_filtered", "rs_edge_join", "rs_containment",
              "rs_pairset_finalize", "rs_estimate_grid", "exclusive_scan_gpu", "merge_and_deduplicate_pairs_gpu",
              "compact_hash_table_pairs", "count_hits_gpu", "compact_hits_gpu", "estimateOverlapSelectivity",
              "estimateIntersectionSelectivity"]:
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB_PATH], stdout=subprocess.PIPE, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"not exported: {missing}"
    for n in declared_functions():
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"
        getattr(lib, n)


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
