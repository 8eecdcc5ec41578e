"""Regenerate the golden fixtures in tests/golden/ (run on a machine with the reference sources).

Two kinds of fixtures:

* reference fixtures -- outputs of the reference's own host code, compiled from its
  sources by oracle/ref_build.py into oracle/_ref/ref_driver:
    EdgePreprocessor::extractEdges   (preprocess/src/EdgePreprocessor.cpp:41-119)
    RaySpace::IO::writeBinaryFile    (common/include/BinaryIO.h:35-102)
    loadPointDataset                 (query/src/runtime/PointIO.cpp:32-92)
    BoundingBox::createBoxMesh       (query/src/geometry/BoundingBox.cpp:4-50)
    generateGridStats                (preprocess/src/preprocess_dataset.cpp:37-181)
    PerformanceTimer JSON            (query/src/timer.cpp:124-192)
  They pin the Python restatements (rayspace3d_gb300/synth.py, formats.py) and the
  oracle's box mesh.
* oracle fixtures -- the CPU oracle's answers for small seeded cases (point-in-mesh,
  overlap and intersection joins, estimator), which the GPU parity tests also check.

Usage: python tests/golden/make_golden.py
"""
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import bind, ref_build  # noqa: E402
from rayspace3d_gb300 import formats, synth  # noqa: E402


def write_in(path, V, I, T, grid=None):
    with open(path, "wb") as f:
        f.write(struct.pack("<QQ", len(V), len(I)))
        f.write(np.ascontiguousarray(V, "<f4").tobytes())
        f.write(np.ascontiguousarray(I, "<u4").tobytes())
        f.write(np.ascontiguousarray(T, "<i4").tobytes())
        if grid is None:
            f.write(b"\x00")
        else:
            f.write(b"\x01")
            f.write(struct.pack("<3f3f3I", *grid.min_bound, *grid.max_bound, *grid.resolution))
            f.write(np.ascontiguousarray(grid.cells).tobytes())


def read_vecs(path, dtypes):
    """Vectors written by ref_driver: u64 element count then the elements; dtypes are
    (numpy dtype, scalars per element), e.g. ("<f4", 3) for float3."""
    buf = open(path, "rb").read()
    pos = 0
    out = []
    for dt, width in dtypes:
        (n,) = struct.unpack_from("<Q", buf, pos)
        pos += 8
        a = np.frombuffer(buf, dtype=dt, count=n * width, offset=pos).copy()
        pos += n * width * np.dtype(dt).itemsize
        out.append(a)
    return out


def edge_cases():
    """Meshes for the edge-extraction fixture: shared edges across objects, duplicated
    vertices, coordinates next to the 1e-5 quantisation boundary."""
    cases = {}
    g = synth.cube_grid(2, 2, 1)
    cases["cube_grid"] = (g.vertices, g.indices, g.tri2obj)
    rng = np.random.default_rng(3)
    V, I, T = synth.assemble_uniform(1, np.array([1.0, 0.7, 1.3]), synth.random_rotations(rng, 3),
                                     rng.uniform(0, 3, size=(3, 3)))
    cases["spheres"] = (V, I, T)
    v = rng.uniform(-2, 2, size=(40, 3)).astype(np.float32)
    v[::5] = np.round(v[::5] * 1e5) / 1e5 + np.float32(0.5e-5)  # half-way quantisation cases
    f = rng.integers(0, 40, size=(60, 3)).astype(np.uint32)
    t = rng.integers(0, 4, size=60).astype(np.int32)
    cases["soup"] = (v, f, t)
    return cases


def main():
    drv = ref_build.build()
    tmp = tempfile.mkdtemp()
    out = {}
    # 1. edge extraction
    for name, (V, I, T) in edge_cases().items():
        p_in = os.path.join(tmp, name + ".bin")
        p_out = os.path.join(tmp, name + ".edges")
        write_in(p_in, V, I, T)
        subprocess.run([drv, "edges", p_in, p_out], check=True, stdout=subprocess.DEVNULL)
        s, e, off, cnt, src = read_vecs(p_out, [("<f4", 3), ("<f4", 3), ("<i4", 1), ("<i4", 1), ("<i4", 1)])
        out[f"edges_{name}_V"] = np.asarray(V, np.float32)
        out[f"edges_{name}_I"] = np.asarray(I, np.uint32)
        out[f"edges_{name}_T"] = np.asarray(T, np.int32)
        out[f"edges_{name}_starts"] = s.reshape(-1, 3)
        out[f"edges_{name}_ends"] = e.reshape(-1, 3)
        out[f"edges_{name}_offsets"] = off
        out[f"edges_{name}_counts"] = cnt
        out[f"edges_{name}_sources"] = src
    # 2. .pre written by the reference writer (edges by the reference, grid by the restatement)
    A, _ = synth.overlap_workload(n_objects=6, level=1, world=10.0, seed=4, grid_resolution=4)
    p_in = os.path.join(tmp, "pre.bin")
    p_pre = os.path.join(HERE, "ref_small.pre")
    write_in(p_in, A.vertices, A.indices, A.tri2obj, A.grid)
    subprocess.run([drv, "prewrite", p_in, p_pre], check=True, stdout=subprocess.DEVNULL)
    # 3. points parsed by the reference parser
    p_txt = os.path.join(HERE, "points.wkt")
    with open(p_txt, "w") as f:
        f.write("# comment line\n\nPOINT (1 2 3)\nPOINT Z (-0.5 2.25 1e-3)\n  POINT(4.000001 5 6)\n")
        f.write("7 8 9\n-1.5 -2.5 -3.5\nLINESTRING (1 2, 3 4)\nPOINT (0.1 0.2 0.3)\n1e5 2 3\n")
    p_pts = os.path.join(tmp, "points.bin")
    subprocess.run([drv, "points", p_txt, p_pts], check=True, stdout=subprocess.DEVNULL)
    out["points"] = read_vecs(p_pts, [("<f4", 3)])[0].reshape(-1, 3)
    # long lines (split by the reader's 1023-byte fgets pieces), CR and CRLF endings, tabs
    p_txt2 = os.path.join(HERE, "points_tricky.wkt")
    with open(p_txt2, "wb") as f:
        f.write(b"POINT (1 2 3)\r\n\tPOINT Z (4 5 6)\n")
        f.write(b"POINT (" + b"7" * 1030 + b" 8 9)\n")
        f.write(b" " * 1020 + b"POINT (10 11 12)\n")
        f.write(b"-1 -2 -3\r-4 -5 -6\n")
        f.write(b"1.5e2 2.5e-1 3\n#POINT (0 0 0)\n")
        f.write(b"POINT(13 14 15)")
    p_pts2 = os.path.join(tmp, "points2.bin")
    subprocess.run([drv, "points", p_txt2, p_pts2], check=True, stdout=subprocess.DEVNULL)
    out["points_tricky"] = read_vecs(p_pts2, [("<f4", 3)])[0].reshape(-1, 3)
    # 4. bounding-box mesh
    g, _ = synth.pim_workload(10, level=2)
    p_in = os.path.join(tmp, "box.bin")
    p_box = os.path.join(tmp, "box.out")
    write_in(p_in, g.vertices, g.indices, g.tri2obj)
    subprocess.run([drv, "box", p_in, p_box], check=True, stdout=subprocess.DEVNULL)
    bv, bi, bo = read_vecs(p_box, [("<f4", 3), ("<u4", 3), ("<i4", 1)])
    out["box_V_in"] = g.vertices
    out["box_vertices"] = bv.reshape(-1, 3)
    out["box_indices"] = bi.reshape(-1, 3)
    # 5. grid statistics: fixed world, bounds from the data, objects partly outside the world
    rng = np.random.default_rng(11)
    G = synth.sphere_set(60, 1, 0.3, 1.5, 8.0, rng, edges=False)
    grid_cases = {"fixed": (A, 4, 10.0), "auto": (G, 8, -1.0), "outside": (G, 5, 6.0)}
    for name, (geo, res, world) in grid_cases.items():
        p_in = os.path.join(tmp, f"grid_{name}.bin")
        p_out = os.path.join(tmp, f"grid_{name}.out")
        write_in(p_in, geo.vertices, geo.indices, geo.tri2obj)
        subprocess.run([drv, "grid", p_in, p_out, str(res), repr(world)], check=True, stdout=subprocess.DEVNULL)
        buf = open(p_out, "rb").read()
        out[f"grid_{name}_V"] = np.asarray(geo.vertices, np.float32)
        out[f"grid_{name}_I"] = np.asarray(geo.indices, np.uint32)
        out[f"grid_{name}_T"] = np.asarray(geo.tri2obj, np.int32)
        out[f"grid_{name}_params"] = np.array([res, world], np.float64)
        out[f"grid_{name}_bounds"] = np.frombuffer(buf, "<f4", 6, 0).copy()
        out[f"grid_{name}_res"] = np.frombuffer(buf, "<u4", 3, 24).copy()
        (n,) = struct.unpack_from("<Q", buf, 36)
        out[f"grid_{name}_cells"] = np.frombuffer(buf, formats.GRID_CELL_DTYPE, n, 44).copy()
    # 6. timer JSON (manual measurements and counters have fixed values)
    p_json = os.path.join(HERE, "timer_reference.json")
    subprocess.run([drv, "timer", p_json], check=True, stdout=subprocess.DEVNULL)

    # Oracle fixtures.
    g, pts = synth.pim_workload(4000, level=3, seed=0)
    out["pim_V"], out["pim_I"], out["pim_T"], out["pim_pts"] = g.vertices, g.indices, g.tri2obj, pts
    out["pim_z"] = bind.pim(g.vertices, g.indices, g.tri2obj, pts)
    out["pim_x"] = bind.pim(g.vertices, g.indices, g.tri2obj, pts, direction=(1.0, 0.0, 0.0))
    out["pim_filtered"] = bind.pim(g.vertices, g.indices, g.tri2obj, pts, filtered=True)
    cg = synth.cube_grid(3, 2, 2)
    cpts = synth.snapped_points(cg, 3000, np.random.default_rng(5), frac_snapped=0.5)
    out["cubes_V"], out["cubes_I"], out["cubes_T"], out["cubes_pts"] = cg.vertices, cg.indices, cg.tri2obj, cpts
    out["cubes_z"] = bind.pim(cg.vertices, cg.indices, cg.tri2obj, cpts)
    A, B = synth.overlap_workload(n_objects=60, level=1, world=8.0, seed=9, grid_resolution=8)
    formats.write_pre(os.path.join(HERE, "join_A.pre"), A)
    formats.write_pre(os.path.join(HERE, "join_B.pre"), B)
    out["join_overlap"] = bind.overlap_join(A, B)
    out["join_intersection"] = bind.intersection_join(A, B)
    est, raw = bind.estimate_pairs(A.grid, B.grid)
    meta = {"join_estimate": est, "join_estimate_raw": raw,
            "generator": "tests/golden/make_golden.py", "reference_driver": "oracle/_ref/ref_driver"}
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
