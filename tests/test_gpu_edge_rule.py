"""The engine's edge-ray hit rule (rs_pairset_set_edge_rule) and parity iteration cap
against the oracle, which tests/test_edge_rule_cpu.py pins to the reference's loops run
literally: edges crossing 240 and 400 faces (the 100-trace cap, the deferred long path of
edges with more than 4 crossings, one warp per edge up to 256 crossings and the one-thread
loop beyond), coincident and near-coincident faces of different
objects (the 1e-6 and 2e-4 steps), through rs_edge_join, rs_overlap_join (broad phase on
and off), the batched launch and raytracer_intersection_estimated's
--overlap-max-iterations.  Pair sets must match bit for bit."""
import ctypes
import os
import subprocess

import numpy as np
import pytest
import torch

import edge_cases as ec
from oracle import bind
from rayspace3d_gb300 import _lib, api, build, formats, synth
from rayspace3d_gb300.formats import Geometry

pytestmark = pytest.mark.gpu


def _segments_geom(A, segs):
    return api.DeviceGeometry(Geometry(A.vertices, A.indices, A.tri2obj, total_triangles=len(A.indices), edges=segs))


@pytest.mark.parametrize("rule", ec.RULES)
@pytest.mark.parametrize("name", sorted(ec.CASES))
def test_edge_join_rule(cuda, name, rule):
    A, B, segs = ec.CASES[name]()
    bb = api.Bvh(api.DeviceGeometry(B))
    ps = api.PairSet(1 << 12)
    ps.set_edge_rule(*rule)
    api.edge_join(bb, _segments_geom(A, segs), ps)
    got = ps.finalize().cpu().numpy().astype(np.uint64)
    want = bind.edge_join(segs, B.vertices, B.indices, B.tri2obj, max_hits=rule[0], next_float=rule[1])
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("cull", [1, 0])
@pytest.mark.parametrize("rule", ec.RULES)
@pytest.mark.parametrize("name", sorted(ec.CASES))
def test_overlap_join_rule(cuda, name, rule, cull):
    A, B, _ = ec.CASES[name]()
    L = _lib.load()
    ba, bb = api.Bvh(api.DeviceGeometry(A)), api.Bvh(api.DeviceGeometry(B))
    ps = api.PairSet(1 << 12)
    ps.set_edge_rule(*rule)
    L.rs_set_overlap_cull(cull)
    try:
        api.overlap_join(ba, bb, ps)
    finally:
        L.rs_set_overlap_cull(1)
    got = ps.finalize().cpu().numpy().astype(np.uint64)
    np.testing.assert_array_equal(got, bind.overlap_join(A, B, max_hits=rule[0], next_float=rule[1]))


def test_edge_rule_default_and_growth(cuda):
    # The default rule is the overlap loop's (100, t + 1e-6); it survives table growth.
    A, B, _ = ec.slab_stack()
    ba, bb = api.Bvh(api.DeviceGeometry(A)), api.Bvh(api.DeviceGeometry(B))
    ps = api.PairSet(4)  # grows inside rs_overlap_join
    api.overlap_join(ba, bb, ps)
    np.testing.assert_array_equal(ps.finalize().cpu().numpy().astype(np.uint64), bind.overlap_join(A, B))
    ps2 = api.PairSet(4)
    ps2.set_edge_rule(1000, False)
    api.overlap_join(ba, bb, ps2)
    assert len(ps2.finalize()) == 120


def test_edge_rule_batched(cuda):
    L = _lib.load()
    A, B, segs = ec.slab_stack()
    bb = api.Bvh(api.DeviceGeometry(B))
    src = _segments_geom(A, segs)
    ps = api.PairSet(1 << 12)
    h = ctypes.c_void_p()
    assert L.rs_batch_create(ctypes.byref(h)) == 0
    try:
        e = src.edge_ptrs()
        assert L.rs_batch_add_edges(h, bb.handle, *e, src.nE, 0, ps.handle, None) == 0
        s = torch.cuda.current_stream()
        for _ in range(2):  # capture, then replay
            ps.clear()
            assert L.rs_batch_submit(h, ctypes.c_void_p(s.cuda_stream)) == 0
            assert L.rs_batch_wait(h, None) == 0
            got = ps.finalize().cpu().numpy().astype(np.uint64)
            np.testing.assert_array_equal(got, bind.edge_join(segs, B.vertices, B.indices, B.tri2obj))
    finally:
        L.rs_batch_destroy(h)


@pytest.mark.parametrize("filtered", [False, True])
@pytest.mark.parametrize("direction", [(0.0, 0.0, 1.0), (0.0, 0.6, 0.8)])
def test_pim_iteration_cap(cuda, direction, filtered):
    from test_edge_rule_cpu import tall_box_points
    g, pts, want = tall_box_points()
    bvh = api.Bvh(api.DeviceGeometry(g))
    obj, inside = api.point_in_mesh(bvh, torch.from_numpy(pts).cuda(), direction=direction, filtered=filtered)
    ref = bind.pim(g.vertices, g.indices, g.tri2obj, pts, direction=direction, filtered=filtered)
    np.testing.assert_array_equal(obj.cpu().numpy(), ref)
    if direction == (0.0, 0.0, 1.0):
        assert ref.tolist() == want


@pytest.mark.parametrize("max_iters", [100, 1000])
def test_cli_overlap_max_iterations(cuda, tmp_path, max_iters):
    A, B, _ = ec.slab_stack()
    A = synth.box_set([((-0.5, 0.30, -0.52), (6.5, 0.32, -0.50))], grid_resolution=8)
    B = synth.box_set([((0.05 * i, -1.0, -1.0), (0.05 * i + 0.01, 1.0, 1.0)) for i in range(120)], grid_resolution=8)
    formats.write_pre(str(tmp_path / "a.pre"), A)
    formats.write_pre(str(tmp_path / "b.pre"), B)
    r = subprocess.run([os.path.join(build.BIN, "raytracer_intersection_estimated"), "--mesh1", "a.pre", "--mesh2",
                        "b.pre", "--output", "t.json", "--overlap-max-iterations", str(max_iters)],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = (tmp_path / "intersection_pairs.csv").read_text().strip().splitlines()[1:]
    got = np.array(sorted((int(a) << 32) | int(b) for a, b in (x.split(",") for x in rows)), np.uint64)
    want = bind.intersection_join(A, B, max_hits=max_iters)
    np.testing.assert_array_equal(got, want)
    assert len(want) == (100 if max_iters == 100 else 120)
