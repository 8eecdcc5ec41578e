"""GPU input preparation (rs_extract_edges) against the reference's own edge payloads
(golden fixtures written by EdgePreprocessor::extractEdges compiled from the reference
sources) and, at larger sizes and on edge cases, against the CPU restatement that those
fixtures pin (synth.extract_edges).  Every comparison is bit-exact."""
import numpy as np
import pytest
import torch

from rayspace3d_gb300 import api, gen, synth

pytestmark = pytest.mark.gpu


def _gpu_edges(V, I, T):
    dV = torch.from_numpy(np.ascontiguousarray(V, np.float32)).cuda()
    dI = torch.from_numpy(np.ascontiguousarray(I, np.uint32).view(np.int32)).cuda()
    dT = torch.from_numpy(np.ascontiguousarray(T, np.int32)).cuda()
    return [t.cpu().numpy() for t in api.extract_edges(dV, dI, dT)]


def _assert_same(got, want):
    s, e, off, cnt, src = got
    np.testing.assert_array_equal(s.view(np.uint32), np.asarray(want[0], np.float32).reshape(-1, 3).view(np.uint32))
    np.testing.assert_array_equal(e.view(np.uint32), np.asarray(want[1], np.float32).reshape(-1, 3).view(np.uint32))
    np.testing.assert_array_equal(off, want[2])
    np.testing.assert_array_equal(cnt, want[3])
    np.testing.assert_array_equal(src, want[4])


@pytest.fixture(scope="module")
def golden():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))


@pytest.mark.parametrize("case", ["cube_grid", "spheres", "soup"])
def test_extract_edges_matches_reference_fixtures(cuda, golden, case):
    p = f"edges_{case}_"
    got = _gpu_edges(golden[p + "V"], golden[p + "I"], golden[p + "T"])
    _assert_same(got, [golden[p + k] for k in ("starts", "ends", "offsets", "counts", "sources")])


def _want(V, I, T):
    w = synth.extract_edges(V, I, T)
    return [w.starts, w.ends, w.offsets, w.counts, w.sources]


def test_extract_edges_instanced_sets(cuda):
    """Sphere sets as the query path sees them (many objects, shared vertices)."""
    rng = np.random.default_rng(7)
    g = synth.sphere_set(400, 2, 0.3, 2.0, 30.0, rng, edges=False)
    _assert_same(_gpu_edges(g.vertices, g.indices, g.tri2obj), _want(g.vertices, g.indices, g.tri2obj))


def test_extract_edges_soup_with_skipped_triangles_and_wide_keys(cuda):
    """Out-of-range indices (triangle skipped), coordinates spanning +-1e6 (three key
    words), points on the 1e-5 rounding half-way, repeated objects on one edge."""
    rng = np.random.default_rng(11)
    nV = 3000
    V = rng.uniform(-1e6, 1e6, size=(nV, 3)).astype(np.float32)
    V[::7] = (np.round(V[::7].astype(np.float64) * 1e5) / 1e5 + 0.5e-5).astype(np.float32)
    V[1::9] = rng.uniform(-2, 2, size=V[1::9].shape).astype(np.float32)
    I = rng.integers(0, nV, size=(20000, 3)).astype(np.uint32)
    I[::97, 1] = nV + 5  # skipped by the reference
    T = rng.integers(0, 6, size=len(I)).astype(np.int32)
    _assert_same(_gpu_edges(V, I, T), _want(V, I, T))


def test_extract_edges_degenerate_long_runs(cuda):
    """All vertices quantise to a handful of points: runs of thousands of records and many
    repeated sources on each edge."""
    rng = np.random.default_rng(5)
    base = rng.uniform(-1, 1, size=(4, 3))
    V = (base[rng.integers(0, 4, 5000)] + rng.uniform(-4e-6, 4e-6, size=(5000, 3))).astype(np.float32)
    I = rng.integers(0, 5000, size=(30000, 3)).astype(np.uint32)
    T = rng.integers(0, 50, size=len(I)).astype(np.int32)
    _assert_same(_gpu_edges(V, I, T), _want(V, I, T))


def test_extract_edges_empty_and_all_skipped(cuda):
    V = np.zeros((3, 3), np.float32)
    out = _gpu_edges(V, np.zeros((0, 3), np.uint32), np.zeros(0, np.int32))
    assert all(len(a) == 0 for a in out)
    out = _gpu_edges(V, np.array([[0, 1, 9]], np.uint32), np.zeros(1, np.int32))
    assert all(len(a) == 0 for a in out)


def test_extract_edges_generator_scale(cuda):
    """A 2000-object intersection set (icospheres of levels 1-3, ~1.1 M triangles) built on
    the device, extracted on the device, against the restatement on the host copy."""
    A, _, _ = gen.intersection_sets(2000, seed=3, world=2000.0 * (2000 / 100_000) ** (1 / 3), levels=(1, 2, 3))
    got = [t.cpu().numpy() for t in api.extract_edges(A.V, A.I, A.T)]
    g = gen.to_host_geometry(A)
    _assert_same(got, _want(g.vertices, g.indices, g.tri2obj))


# ----------------------------------------------------------------- grid statistics

def _gpu_grid(V, I, T, R, world, n_obj=None):
    import ctypes
    from rayspace3d_gb300 import _lib, formats
    dV = torch.from_numpy(np.ascontiguousarray(V, np.float32)).cuda()
    dI = torch.from_numpy(np.ascontiguousarray(I, np.uint32).view(np.int32)).cuda()
    dT = torch.from_numpy(np.ascontiguousarray(T, np.int32)).cuda()
    cells = torch.empty(R ** 3 * 16, dtype=torch.uint8, device="cuda")
    b = (ctypes.c_float * 6)()
    n_obj = int(T.max()) + 1 if n_obj is None else n_obj
    st = _lib.load().rs_grid_stats(dV.data_ptr(), len(V), dI.data_ptr(), len(I), dT.data_ptr(), n_obj, R, world,
                                   cells.data_ptr(), b, None)
    return st, np.array(b[:], np.float32), cells.cpu().numpy().view(formats.GRID_CELL_DTYPE)


@pytest.mark.parametrize("case", ["fixed", "auto", "outside"])
def test_grid_stats_matches_reference_fixtures(cuda, golden, case):
    """Cells and bounds written by the reference's generateGridStats, bit for bit."""
    p = f"grid_{case}_"
    res, world = golden[p + "params"]
    st, b, cells = _gpu_grid(golden[p + "V"], golden[p + "I"], golden[p + "T"], int(res), float(world))
    assert st == 0
    np.testing.assert_array_equal(b.view(np.uint32), golden[p + "bounds"].view(np.uint32))
    np.testing.assert_array_equal(cells.view(np.uint8), golden[p + "cells"].view(np.uint8))


@pytest.mark.parametrize("shuffle", [False, True])
@pytest.mark.parametrize("world", [60.0, -1.0])
def test_grid_stats_exact_on_sphere_sets(cuda, shuffle, world):
    """Hundreds of objects (several rehashes of the reference's object map), objects stored
    contiguously or with their triangles interleaved, some triangles skipped."""
    rng = np.random.default_rng(9)
    g = synth.sphere_set(700, 1, 0.3, 6.0, 60.0, rng, edges=False)
    V, I, T = g.vertices, g.indices.copy(), g.tri2obj
    if shuffle:
        p = rng.permutation(len(I))
        I, T = I[p], T[p]
    I[::53, 2] = len(V) + 1
    R = 32
    st, b, cells = _gpu_grid(V, I, T, R, world)
    assert st == 0
    want = synth.grid_stats(V, I, T, R, world)
    np.testing.assert_array_equal(b[:3].view(np.uint32), want.min_bound.view(np.uint32))
    np.testing.assert_array_equal(cells.view(np.uint8), want.cells.view(np.uint8))


def test_grid_stats_rejects_object_outside_range(cuda):
    rng = np.random.default_rng(2)
    g = synth.sphere_set(10, 1, 0.3, 1.0, 10.0, rng, edges=False)
    st, _, _ = _gpu_grid(g.vertices, g.indices, g.tri2obj, 8, 10.0, n_obj=5)
    assert st == 2  # RS_ERR_INVALID


# ----------------------------------------------------------------- preprocess_dataset

def _run_pre(tmp_path, src, *flags):
    import json
    import os
    import subprocess
    from rayspace3d_gb300 import build
    exe = os.path.join(build.BIN, "preprocess_dataset")
    out, tj = tmp_path / "out.pre", tmp_path / "timing.json"
    r = subprocess.run([exe, "--dataset", str(src), "--output-geometry", str(out), "--output-timing", str(tj),
                        *flags], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return out.read_bytes(), json.loads(tj.read_text()), r.stdout


def test_preprocess_reproduces_reference_written_file(cuda, tmp_path):
    """ref_small.pre was written by the reference's writer around the reference's edge
    extraction; preprocessing its geometry on the GPU writes the same bytes (the 6 header
    padding bytes aside, which the reference leaves uninitialised)."""
    import os
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_small.pre")
    got, timing, out = _run_pre(tmp_path, src, "--generate-grid", "--grid-resolution", "4", "--world-size", "10")
    want = open(src, "rb").read()
    assert len(got) == len(want)
    assert got[58:64] == b"\0" * 6
    assert got[:58] == want[:58] and got[64:] == want[64:]
    assert list(timing["phases"]) == ["loading dataset_1", "generating grid statistics_1", "extracting edges_1",
                                      "writing geometry data_1"]
    assert "counters" not in timing and timing["total"]["duration_us"] > 0
    assert "Extracted " in out and "=== Preprocessing Complete ===" in out


@pytest.mark.parametrize("interleave", [False, True])
def test_preprocess_matches_host_restatement(cuda, tmp_path, interleave):
    """A 2000-object set (grid with bounds from the data, triangles of different objects
    interleaved or not): the GPU-preprocessed file equals the host restatement's, byte for
    byte."""
    from rayspace3d_gb300 import formats
    rng = np.random.default_rng(21)
    g = synth.sphere_set(2000, 2, 0.3, 3.0, 200.0, rng, edges=False)
    V, I, T = g.vertices, g.indices, g.tri2obj
    if interleave:
        p = rng.permutation(len(I))
        I, T = I[p], T[p]
    src = tmp_path / "in.pre"
    formats.write_pre(str(src), formats.Geometry(V, I, T, total_triangles=len(I)))
    got, _, _ = _run_pre(tmp_path, src, "--generate-grid", "--grid-resolution", "64")
    want_path = tmp_path / "want.pre"
    formats.write_pre(str(want_path), synth.make_geometry(V, I, T, edges=True, grid_resolution=64, world_size=-1.0))
    assert got == want_path.read_bytes()


def test_preprocess_refuses_other_loaders(cuda, tmp_path):
    import os
    import subprocess
    from rayspace3d_gb300 import build
    obj = tmp_path / "x.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    r = subprocess.run([os.path.join(build.BIN, "preprocess_dataset"), "--dataset", str(obj)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 1 and "Could not determine loader" in r.stderr


def test_extract_edges_capacity_overflow_reports_sizes(cuda):
    import ctypes
    from rayspace3d_gb300 import _lib
    rng = np.random.default_rng(1)
    g = synth.sphere_set(20, 1, 0.5, 1.0, 10.0, rng, edges=False)
    want = synth.extract_edges(g.vertices, g.indices, g.tri2obj)
    dV = torch.from_numpy(np.ascontiguousarray(g.vertices, np.float32)).cuda()
    dI = torch.from_numpy(np.ascontiguousarray(g.indices, np.uint32).view(np.int32)).cuda()
    dT = torch.from_numpy(np.ascontiguousarray(g.tri2obj, np.int32)).cuda()
    cap = 10
    bufs = [torch.zeros(cap * 3, dtype=torch.float32, device="cuda") for _ in range(2)] + \
           [torch.zeros(cap, dtype=torch.int32, device="cuda") for _ in range(3)]
    nE, nS = ctypes.c_uint64(), ctypes.c_uint64()
    st = _lib.load().rs_extract_edges(dV.data_ptr(), len(g.vertices), dI.data_ptr(), len(g.indices), dT.data_ptr(),
                                      *[b.data_ptr() for b in bufs], cap, ctypes.byref(nE), ctypes.byref(nS), None)
    assert st == 4  # RS_ERR_OUTPUT_OVERFLOW
    assert nE.value == len(want.starts) and nS.value == len(want.sources)
    assert all(int(b.abs().sum().item()) == 0 for b in bufs)  # outputs untouched


def test_grid_stats_without_triangles(cuda):
    V = np.array([[0, 0, 0], [2, 3, 4], [1, 1, 1]], np.float32)
    st, b, cells = _gpu_grid(V, np.zeros((0, 3), np.uint32), np.zeros(0, np.int32), 4, -1.0, n_obj=0)
    assert st == 0
    np.testing.assert_array_equal(b, np.array([0, 0, 0, 2, 3, 4], np.float32))
    assert cells.view(np.uint8).sum() == 0


def test_preprocess_shuffle_moves_objects_rigidly(cuda, tmp_path):
    """--shuffle: one random translation per object (as the reference, not reproducible);
    triangles and objects unchanged, each object's vertices moved by one vector in
    [-15, 15]^3, edges and grid derived from the moved geometry."""
    from rayspace3d_gb300 import formats
    rng = np.random.default_rng(3)
    g = synth.sphere_set(50, 1, 0.5, 1.0, 40.0, rng, edges=False)
    src = tmp_path / "in.pre"
    formats.write_pre(str(src), formats.Geometry(g.vertices, g.indices, g.tri2obj, total_triangles=len(g.indices)))
    out, _, _ = _run_pre(tmp_path, src, "--shuffle")
    h = formats.read_pre(str(tmp_path / "out.pre"))
    np.testing.assert_array_equal(h.indices, g.indices)
    np.testing.assert_array_equal(h.tri2obj, g.tri2obj)
    d = h.vertices.astype(np.float64) - g.vertices.astype(np.float64)
    for o in range(50):
        vs = np.unique(g.indices[g.tri2obj == o])
        assert np.all(np.abs(d[vs] - d[vs[0]]) < 1e-4) and np.all(np.abs(d[vs[0]]) <= 15.0 + 1e-4)
    e = synth.extract_edges(h.vertices, h.indices, h.tri2obj)
    np.testing.assert_array_equal(h.edges.offsets, e.offsets)
    np.testing.assert_array_equal(h.edges.sources, e.sources)
