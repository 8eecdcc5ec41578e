"""GPU parity against the committed golden fixtures, the tracked containment, and the
drop-in executables end to end (files in, CSV/JSON out) against the oracle answers.

Every comparison is exact: first-hit objects, pair sets, per-source candidate counts and
crossed-triangle counts are integers.
"""
import csv
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, build, formats

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLD, "golden.npz"))


@pytest.fixture(scope="module")
def meta():
    with open(os.path.join(GOLD, "golden_meta.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def join_sets():
    return formats.read_pre(os.path.join(GOLD, "join_A.pre")), formats.read_pre(os.path.join(GOLD, "join_B.pre"))


def _geom(g, prefix):
    return formats.Geometry(g[prefix + "V"], g[prefix + "I"], g[prefix + "T"], total_triangles=len(g[prefix + "I"]))


def _gpu_pim(geo, pts, direction=(0.0, 0.0, 1.0), filtered=False):
    bvh = api.Bvh(api.DeviceGeometry(geo))
    obj, _ = api.point_in_mesh(bvh, torch.from_numpy(np.ascontiguousarray(pts)).cuda(), direction=direction,
                               filtered=filtered)
    torch.cuda.synchronize()
    return obj.cpu().numpy()


def test_pim_matches_golden(cuda, golden):
    geo = _geom(golden, "pim_")
    pts = golden["pim_pts"]
    np.testing.assert_array_equal(_gpu_pim(geo, pts), golden["pim_z"])
    np.testing.assert_array_equal(_gpu_pim(geo, pts, direction=(1.0, 0.0, 0.0)), golden["pim_x"])
    np.testing.assert_array_equal(_gpu_pim(geo, pts, filtered=True), golden["pim_filtered"])
    cubes = _geom(golden, "cubes_")
    np.testing.assert_array_equal(_gpu_pim(cubes, golden["cubes_pts"]), golden["cubes_z"])


def test_joins_match_golden(cuda, golden, meta, join_sets):
    A, B = join_sets
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ps = api.PairSet(1 << 12)
    api.overlap_join(ba, bb, ps)
    np.testing.assert_array_equal(np.sort(ps.finalize().cpu().numpy().astype(np.uint64)), golden["join_overlap"])
    ps.clear()
    api.overlap_join(ba, bb, ps, with_containment=True)
    np.testing.assert_array_equal(np.sort(ps.finalize().cpu().numpy().astype(np.uint64)),
                                  golden["join_intersection"])
    est, raw = api.estimate_pairs(da, db)
    assert est == meta["join_estimate"]
    assert raw == pytest.approx(meta["join_estimate_raw"], rel=1e-5)


def _tracked(bvh, src, max_targets, swap=0, capacity=None):
    L = _lib.load()
    ds = api.DeviceGeometry(src)
    n_obj = src.num_objects
    cap = n_obj if capacity is None else capacity
    ids = torch.full((max(cap, 1) * max_targets,), 7, dtype=torch.int32, device="cuda")
    hits = torch.full_like(ids, 7)
    cand = torch.full((max(cap, 1),), 7, dtype=torch.int32, device="cuda")
    ps = api.PairSet(1 << 12)
    L.rs_pairset_set_tracking(ps.handle, 1)
    rc = L.rs_containment_tracked(bvh.handle, ds.V.data_ptr(), ds.nV, ds.I.data_ptr(), ds.nF, ds.T.data_ptr(), swap,
                                  ps.handle, max_targets, ids.data_ptr(), hits.data_ptr(), cand.data_ptr(), cap, None)
    torch.cuda.synchronize()
    return rc, ps, ids.cpu().numpy().reshape(-1, max_targets), hits.cpu().numpy().reshape(-1, max_targets), \
        cand.cpu().numpy()


def test_containment_tracked_matches_oracle(cuda, join_sets):
    """Per-source candidate counts, odd-parity targets and their crossed-triangle counts
    (PairHitTracking.h:31-150 diagnostics) equal the oracle's; the pairs equal plain
    containment; the counters count rays, crossings and distinct targets."""
    A, B = join_sets
    bb = api.Bvh(api.DeviceGeometry(B))
    rc, ps, ids, hits, cand = _tracked(bb, A, max_targets=8)
    assert rc == 0
    want_cand, want_keys, want_hits = bind.containment_diag(A, B.vertices, B.indices, B.tri2obj)
    np.testing.assert_array_equal(cand.astype(np.uint32), want_cand)
    got = sorted((s << 32 | int(t), int(h)) for s in range(len(cand)) for t, h in zip(ids[s], hits[s]) if t >= 0)
    assert [k for k, _ in got] == [int(k) for k in want_keys]
    assert [h for _, h in got] == [int(h) for h in want_hits]
    keys = np.sort(ps.finalize().cpu().numpy().astype(np.uint64))
    np.testing.assert_array_equal(keys, bind.containment(A, B.vertices, B.indices, B.tri2obj))
    c = np.zeros(8, np.uint64)
    assert _lib.load().rs_pairset_counters(ps.handle, c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None) == 0
    assert int(c[4]) == A.num_objects
    assert int(c[6]) == int(want_cand.sum())
    assert int(c[5]) >= int(want_hits.sum())
    assert int(c[0]) >= len(keys)


def test_containment_tracked_capacity_and_truncation(cuda, join_sets):
    A, B = join_sets
    bb = api.Bvh(api.DeviceGeometry(B))
    rc, *_ = _tracked(bb, A, max_targets=4, capacity=A.num_objects - 1)
    assert rc == _lib.RS_ERR_OUTPUT_OVERFLOW
    # one slot per source: the pair set stays complete, the per-source list keeps the first
    rc, ps, ids, hits, cand = _tracked(bb, A, max_targets=1)
    assert rc == 0
    want_cand, want_keys, _ = bind.containment_diag(A, B.vertices, B.indices, B.tri2obj)
    np.testing.assert_array_equal(cand.astype(np.uint32), want_cand)
    odd_sources = set(int(k) >> 32 for k in want_keys)
    assert set(np.nonzero(ids[:, 0] >= 0)[0].tolist()) == odd_sources
    np.testing.assert_array_equal(np.sort(ps.finalize().cpu().numpy().astype(np.uint64)),
                                  bind.containment(A, B.vertices, B.indices, B.tri2obj))


# ---------------------------------------------------------------------- executables

@pytest.fixture(scope="module")
def cli():
    build.build_lib()
    build.build_cli()
    return lambda app: os.path.join(build.BIN, app)


def _run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, f"{cmd[0]} exited {r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}"
    return r.stdout


def _read_csv(path):
    with open(path) as f:
        rows = list(csv.reader(f))
    return rows[0], rows[1:]


def _timing(path):
    with open(path) as f:
        return json.load(f)


def test_cli_raytracer(cuda, cli, golden, tmp_path):
    geo = _geom(golden, "pim_")
    formats.write_pre(str(tmp_path / "g.pre"), geo)
    pts = golden["pim_pts"]
    formats.write_points_wkt(str(tmp_path / "p.wkt"), pts)
    out = _run([cli("raytracer"), "--geometry", "g.pre", "--points", "p.wkt", "--output", "t.json", "--runs", "2",
                "--warmup-runs", "1"], tmp_path)
    head, rows = _read_csv(tmp_path / "ray_results.csv")
    assert head == ["pointId", "polygonId"]
    want = golden["pim_z"]
    ids = np.nonzero(want >= 0)[0]
    assert [(int(a), int(b)) for a, b in rows] == [(int(i), int(want[i])) for i in ids]
    assert f"Points INSIDE polygons:  {len(ids)}" in out
    t = _timing(tmp_path / "t.json")
    assert "data reading_1" in t["phases"] and "build index_1" in t["phases"] and t["total"]["duration_us"] > 0


def test_cli_filter_refine(cuda, cli, golden, tmp_path):
    geo = _geom(golden, "pim_")
    formats.write_pre(str(tmp_path / "g.pre"), geo)
    formats.write_points_wkt(str(tmp_path / "p.wkt"), golden["pim_pts"])
    _run([cli("raytracer_filter_refine"), "--geometry", "g.pre", "--points", "p.wkt", "--output", "t.json"], tmp_path)
    _, rows = _read_csv(tmp_path / "ray_results.csv")
    want = golden["pim_filtered"]
    assert sorted((int(a), int(b)) for a, b in rows) == [(int(i), int(want[i])) for i in np.nonzero(want >= 0)[0]]


def _keys(rows):
    return np.array([(int(a) << 32) | int(b) for a, b in rows], dtype=np.uint64)


def test_cli_mesh_overlap(cuda, cli, golden, tmp_path):
    _run([cli("raytracer_mesh_overlap"), "--mesh1", os.path.join(GOLD, "join_A.pre"), "--mesh2",
          os.path.join(GOLD, "join_B.pre"), "--output", "t.json", "--runs", "2"], tmp_path)
    head, rows = _read_csv(tmp_path / "mesh_overlap_results.csv")
    assert head == ["object_id_mesh1", "object_id_mesh2"]
    k = _keys(rows)
    np.testing.assert_array_equal(np.sort(k), golden["join_overlap"])
    # rows ascend by (object_id_mesh2, object_id_mesh1)
    swapped = [(int(b), int(a)) for a, b in rows]
    assert swapped == sorted(swapped)


@pytest.mark.parametrize("app", ["raytracer_overlap_estimated", "raytracer_overlap_direct_estimation"])
def test_cli_overlap_estimated(cuda, cli, golden, meta, tmp_path, app):
    extra = ["--pairs-output", "pairs.csv"] if app.endswith("direct_estimation") else []
    out = _run([cli(app), "--mesh1", os.path.join(GOLD, "join_A.pre"), "--mesh2", os.path.join(GOLD, "join_B.pre"),
                "--output", "t.json"] + extra, tmp_path)
    assert f"Final Estimated Pairs:     {meta['join_estimate']}" in out
    assert f"Unique object pairs: {len(golden['join_overlap'])}" in out
    if extra:
        _, rows = _read_csv(tmp_path / "pairs.csv")
        np.testing.assert_array_equal(np.sort(_keys(rows)), golden["join_overlap"])


def test_cli_intersection_estimated(cuda, cli, golden, meta, tmp_path, join_sets):
    A, B = join_sets
    out = _run([cli("raytracer_intersection_estimated"), "--mesh1", os.path.join(GOLD, "join_A.pre"), "--mesh2",
                os.path.join(GOLD, "join_B.pre"), "--output", "t.json", "--enable-profiling-stats"], tmp_path)
    assert f"Actual Intersection Pairs: {len(golden['join_intersection'])}" in out
    head, rows = _read_csv(tmp_path / "intersection_pairs.csv")
    assert head == ["a_object_id", "b_object_id"]
    k = _keys(rows)
    np.testing.assert_array_equal(k, golden["join_intersection"])      # sorted by (a, b)
    head, rows = _read_csv(tmp_path / "intersection_containment_tracking.csv")
    assert head == ["direction", "source_object_id", "iterations", "candidate_count", "candidate_overflow_events"]
    c1, k1, h1 = bind.containment_diag(A, B.vertices, B.indices, B.tri2obj)
    c2, k2, h2 = bind.containment_diag(B, A.vertices, A.indices, A.tri2obj)
    got1 = [int(r[3]) for r in rows if r[0] == "mesh1_to_mesh2"]
    got2 = [int(r[3]) for r in rows if r[0] == "mesh2_to_mesh1"]
    assert got1 == c1.tolist() and got2 == c2.tolist()
    _, rows = _read_csv(tmp_path / "intersection_pair_hits.csv")
    hits1 = sorted(((int(r[1]) << 32) | int(r[2]), int(r[3])) for r in rows if r[0] == "mesh1_to_mesh2")
    hits2 = sorted(((int(r[1]) << 32) | int(r[2]), int(r[3])) for r in rows if r[0] == "mesh2_to_mesh1")
    assert hits1 == [(int(a), int(b)) for a, b in zip(k1, h1)]
    assert hits2 == [(int(a), int(b)) for a, b in zip(k2, h2)]
    t = _timing(tmp_path / "t.json")
    assert t["counters"]["profile_actual_intersection_pairs"] == len(golden["join_intersection"])
    assert t["counters"]["profile_containment_rays_total"] == A.num_objects + B.num_objects


def _many_targets():
    """A containment ray that crosses 90 distinct target objects: 50 nested cubes around
    the ray origin (one crossing each, odd) and 40 cubes stacked above it (two each)."""
    from rayspace3d_gb300 import synth
    rng = np.random.default_rng(31)
    Vs, Is, Ts = [], [], []
    ids = rng.permutation(90)
    o = np.array([0.1, 0.2, 0.3])
    for k in range(90):
        if k < 50:
            h = 1.0 + 0.5 * k
            lo, hi = o - h + np.array([0.013, 0.007, 0.0]), o + h + np.array([0.013, 0.007, 0.0])
        else:
            z = 200.0 + 2.0 * (k - 50)
            lo, hi = np.array([o[0] - 0.5, o[1] - 0.4, z]), np.array([o[0] + 0.6, o[1] + 0.5, z + 1.0])
        v, f = synth.cube_mesh(lo, hi)
        Is.append(f + np.uint32(8 * k))
        Vs.append(v)
        Ts.append(np.full(12, ids[k], np.int32))
    tgt = formats.Geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts), total_triangles=12 * 90)
    src = formats.Geometry(np.array([o, o + [1, 0, 0], o + [0, 1, 0], [500, 0, 0], [501, 0, 0], [500, 1, 0]],
                                    np.float32),
                           np.array([[0, 1, 2], [3, 4, 5]], np.uint32), np.array([0, 1], np.int32), total_triangles=2)
    return src, tgt, ids


def test_containment_beyond_32_targets(cuda):
    src, tgt, ids = _many_targets()
    bt = api.Bvh(api.DeviceGeometry(tgt))
    for max_targets in (64, 8):
        rc, ps, got_ids, got_hits, cand = _tracked(bt, src, max_targets=max_targets)
        assert rc == 0
        want_cand, want_keys, want_hits = bind.containment_diag(src, tgt.vertices, tgt.indices, tgt.tri2obj)
        assert want_cand.tolist() == [90, 0]
        np.testing.assert_array_equal(cand.astype(np.uint32), want_cand)
        assert sorted(int(k) & 0xFFFFFFFF for k in want_keys) == sorted(ids[:50].tolist())
        keys = np.sort(ps.finalize().cpu().numpy().astype(np.uint64))
        np.testing.assert_array_equal(keys, want_keys)
        listed = [int(t) for t in got_ids[0] if t >= 0]
        assert len(listed) == min(50, max_targets) and set(listed) <= set(ids[:50].tolist())
        assert all(h == 1 for t, h in zip(got_ids[0], got_hits[0]) if t >= 0)
        c = np.zeros(8, np.uint64)
        _lib.load().rs_pairset_counters(ps.handle, c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None)
        assert int(c[4]) == 2 and int(c[5]) == 50 + 2 * 40 and int(c[6]) == 90
    ps = api.PairSet(1 << 10)
    api.containment(bt, api.DeviceGeometry(src), ps, swap=True)
    np.testing.assert_array_equal(np.sort(ps.finalize().cpu().numpy().astype(np.uint64)),
                                  bind.containment(src, tgt.vertices, tgt.indices, tgt.tri2obj, swap=True))


def test_recheck_counters(cuda, golden):
    """Points snapped onto shared cube edges and vertices need the exact path; the counters
    see it, and results stay equal to the oracle's."""
    L = _lib.load()
    cubes = _geom(golden, "cubes_")
    pts = golden["cubes_pts"]
    L.rs_recheck_reset()
    L.rs_recheck_enable(1)
    try:
        got = _gpu_pim(cubes, pts)
    finally:
        L.rs_recheck_enable(0)
    ex, tests = ctypes.c_uint64(), ctypes.c_uint64()
    assert L.rs_recheck_read(ctypes.byref(ex), ctypes.byref(tests)) == 0
    np.testing.assert_array_equal(got, golden["cubes_z"])
    assert tests.value > 0 and ex.value > 0
    assert ex.value <= 3 * tests.value + 3 * 12 * len(pts)
    L.rs_recheck_reset()
    assert L.rs_recheck_read(ctypes.byref(ex), ctypes.byref(tests)) == 0
    assert ex.value == 0 and tests.value == 0


def test_async_builds_on_two_streams(cuda, golden, join_sets):
    """rs_bvh_build_async on two streams, then a join on a third: the engine orders the
    join after both builds; results equal the oracle's."""
    A, B = join_sets
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    torch.cuda.synchronize()
    s1, s2, s3 = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ba = api.Bvh(da, stream=s1, asynchronous=True)
    bb = api.Bvh(db, stream=s2, asynchronous=True)
    ps = api.PairSet(1 << 12, stream=s3)
    api.overlap_join(ba, bb, ps, with_containment=True, stream=s3)
    keys = np.sort(ps.finalize(stream=s3).cpu().numpy().astype(np.uint64))
    np.testing.assert_array_equal(keys, golden["join_intersection"])
    ba.wait()
    bb.wait()
    info = ba.info()
    assert info["triangles"] == len(A.indices)
    np.testing.assert_array_equal(np.array(info["min"], np.float32), A.vertices.min(axis=0))
    # point-in-mesh straight after an asynchronous build on another stream
    geo = _geom(golden, "pim_")
    bp = api.Bvh(api.DeviceGeometry(geo), stream=s1, asynchronous=True)
    obj, _ = api.point_in_mesh(bp, torch.from_numpy(golden["pim_pts"]).cuda(), stream=s2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(obj.cpu().numpy(), golden["pim_z"])


def test_out_of_range_vertex_index(cuda):
    """An index past the vertex array is reported, synchronously by rs_bvh_build and by
    rs_bvh_wait after an asynchronous build (the kernels clamp every index)."""
    L = _lib.load()
    V = torch.tensor([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=torch.float32, device="cuda")
    I = torch.tensor([[0, 1, 2], [0, 1, 7]], dtype=torch.int32, device="cuda")
    T = torch.zeros(2, dtype=torch.int32, device="cuda")
    h = ctypes.c_void_p()
    assert L.rs_bvh_build(V.data_ptr(), 3, I.data_ptr(), 2, T.data_ptr(), 0, ctypes.byref(h), None) == \
        _lib.RS_ERR_INVALID
    assert not h.value
    assert L.rs_bvh_build_async(V.data_ptr(), 3, I.data_ptr(), 2, T.data_ptr(), 0, ctypes.byref(h), None) == 0
    assert L.rs_bvh_wait(h) == _lib.RS_ERR_INVALID
    pts = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    obj = torch.empty(4, dtype=torch.int32, device="cuda")
    assert L.rs_pim(h, pts.data_ptr(), 4, 0.0, 0.0, 1.0, obj.data_ptr(), None, None) == _lib.RS_ERR_INVALID
    assert L.rs_bvh_destroy(h) == 0


@pytest.mark.parametrize("include_overlap", [False, True])
def test_cli_containment(cuda, cli, tmp_path, include_overlap):
    """raytracer_containment on sets with B objects planted inside A objects: strict
    containment pairs (and the overlap pairs) equal the oracle's."""
    from rayspace3d_gb300 import gen
    A, B, planted = gen.intersection_sets(400, seed=8, world=300.0, levels=(1, 2, 3))
    ha, hb = gen.to_host_geometry(A), gen.to_host_geometry(B)
    formats.write_pre(str(tmp_path / "a.pre"), ha)
    formats.write_pre(str(tmp_path / "b.pre"), hb)
    extra = ["--include-overlap-pairs"] if include_overlap else []
    out = _run([cli("raytracer_containment"), "--mesh1", "a.pre", "--mesh2", "b.pre", "--output", "t.json",
                "--runs", "2"] + extra, tmp_path)
    strict, overlap = bind.containment_strict(ha, hb)
    assert f"Containment pairs (B in A): {len(strict)}" in out
    head, rows = _read_csv(tmp_path / "mesh_containment_results.csv")
    if include_overlap:
        assert head == ["a_object_id", "b_object_id", "pair_type"]
        got_c = _keys([r[:2] for r in rows if r[2] == "containment"])
        got_o = _keys([r[:2] for r in rows if r[2] == "overlap"])
        np.testing.assert_array_equal(got_o, overlap)
    else:
        assert head == ["a_object_id", "b_object_id"]
        got_c = _keys(rows)
    np.testing.assert_array_equal(got_c, strict)
    # planted objects that touch nothing else are strict containment pairs
    keys = set(int(k) for k in strict) | set(int(k) for k in overlap)
    assert all(((a << 32) | b) in keys for a, b in planted)
    t = _timing(tmp_path / "t.json")
    assert "build a index_1" in t["phases"] and "query_1" in t["phases"]
