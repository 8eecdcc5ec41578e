"""GPU parity: every engine entry point against the CPU oracle on the same seeded inputs.

Integer/index outputs (containment vectors, first-hit objects, pair sets) must match
bit for bit.  The estimator's raw sum is floating point: |gpu - oracle| <= 1e-5 * |oracle|
(per-cell powf may differ by a few ulp between CUDA and the host libm).
"""
import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu


def _pim(g, pts, direction=(0.0, 0.0, 1.0), filtered=False, leaf=0):
    dg = api.DeviceGeometry(g)
    bvh = api.Bvh(dg, leaf_size=leaf)
    obj, inside = api.point_in_mesh(bvh, torch.from_numpy(np.ascontiguousarray(pts)).cuda(), direction=direction,
                                    filtered=filtered)
    torch.cuda.synchronize()
    return obj.cpu().numpy(), inside.cpu().numpy()


def _check_pim(g, pts, direction=(0.0, 0.0, 1.0), filtered=False, leaf=0):
    got, inside = _pim(g, pts, direction, filtered, leaf)
    want = bind.pim(g.vertices, g.indices, g.tri2obj, pts, direction=direction, filtered=filtered)
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, f"{len(bad)} mismatches, first {bad[:5]}: gpu {got[bad[:5]]} oracle {want[bad[:5]]}"
    assert np.array_equal(inside.astype(bool), want >= 0)
    return want


def test_radix_sort_matches_numpy(cuda):
    from rayspace3d_gb300 import _lib as L
    rng = np.random.default_rng(5)
    cases = [(n, "wide") for n in (1, 7, 3071, 3072, 3073, 4096, 4097, 100_003, 2_000_003)]
    cases += [(1_500_001, "narrow")]
    for n, kind in cases:
        if kind == "wide":
            keys = rng.integers(0, 2 ** 63, size=n, dtype=np.int64)
            keys[: n // 3] = keys[0]  # many duplicates
        else:  # few distinct values in a middle digit range: long runs per digit
            keys = (rng.integers(0, 300, size=n, dtype=np.int64) << 40) | rng.integers(0, 5, size=n, dtype=np.int64)
        t = torch.from_numpy(keys.copy()).cuda()
        out = torch.empty_like(t)
        # merge_and_deduplicate_pairs_gpu sorts the 8-byte records as u64 and uniques them
        cnt = L.load().merge_and_deduplicate_pairs_gpu(t.data_ptr(), n, None, 0, out.data_ptr())
        want = np.unique(keys.view(np.uint64))
        assert cnt == len(want)
        got = t.cpu().numpy().view(np.uint64)[:cnt] if False else out.cpu().numpy().view(np.uint64)[:cnt]
        assert np.array_equal(got, want)


def test_exclusive_scan_compat(cuda):
    rng = np.random.default_rng(1)
    for n in (1, 4095, 4096, 70_001):
        x = rng.integers(0, 1000, size=n).astype(np.int32)
        d_in = torch.from_numpy(x).cuda()
        d_out = torch.empty(n, dtype=torch.int64, device="cuda")
        tot = _lib.load().exclusive_scan_gpu(d_in.data_ptr(), d_out.data_ptr(), n)
        assert tot == int(x.sum())
        want = np.concatenate([[0], np.cumsum(x.astype(np.int64))[:-1]])
        assert np.array_equal(d_out.cpu().numpy(), want)


def test_pim_sphere_plus_z(cuda):
    g, pts = synth.pim_workload(60_000, level=4, seed=0)
    want = _check_pim(g, pts)
    r = np.linalg.norm(pts.astype(np.float64), axis=1)
    assert (want[r < 0.99] == 0).all() and (want[r > 1.0] == -1).all()


def test_pim_sphere_plus_x_and_general_direction(cuda):
    g, pts = synth.pim_workload(30_000, level=3, seed=4)
    a = _check_pim(g, pts, direction=(1.0, 0.0, 0.0))
    b = _check_pim(g, pts, direction=(0.0, 1.0, 0.0))
    d = np.array([0.3, -0.5, 0.8], np.float32)
    d = (d / np.linalg.norm(d)).astype(np.float32)
    c = _check_pim(g, pts, direction=tuple(float(x) for x in d))
    # a closed mesh: inside/outside does not depend on the direction for generic points
    assert (a >= 0).mean() == pytest.approx((b >= 0).mean(), abs=2e-3)
    assert (a >= 0).mean() == pytest.approx((c >= 0).mean(), abs=2e-3)


@pytest.mark.parametrize("leaf", [1, 2, 4, 8])
def test_pim_leaf_sizes(cuda, leaf):
    g, pts = synth.pim_workload(20_000, level=4, seed=2)
    _check_pim(g, pts, leaf=leaf)


def test_pim_degenerate_cubes_and_snapped_points(cuda):
    g = synth.cube_grid(4, 3, 2)
    rng = np.random.default_rng(7)
    pts = synth.snapped_points(g, 40_000, rng, frac_snapped=0.5)
    # also points exactly on grid planes, lines and lattice corners
    lat = rng.integers(0, 5, size=(20_000, 3)).astype(np.float32)
    frac = rng.uniform(0, 4, size=(20_000, 3)).astype(np.float32)
    mask = rng.integers(0, 2, size=(20_000, 3)).astype(bool)
    lattice = np.where(mask, lat, frac).astype(np.float32)
    allpts = np.concatenate([pts, lattice])
    for d in [(0.0, 0.0, 1.0), (1.0, 0.0, 0.0)]:
        _check_pim(g, allpts, direction=d)
    _check_pim(g, allpts, filtered=True)


def test_pim_many_hits_fallback(cuda):
    # 16 nested spheres: rays from the centre region cross more than 8 surfaces.
    Vs, Is, Ts = [], [], []
    v, f = synth.icosphere(3)
    off = 0
    for k in range(16):
        Vs.append((v * (1.0 + 0.05 * k)).astype(np.float32))
        Is.append(f + np.uint32(off))
        Ts.append(np.full(len(f), k, np.int32))
        off += len(v)
    g = synth.make_geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts), edges=False)
    pts = np.random.default_rng(3).uniform(-2, 2, size=(20_000, 3)).astype(np.float32)
    _check_pim(g, pts)


def test_pim_filtered_matches_oracle(cuda):
    g, pts = synth.pim_workload(40_000, level=4, seed=9, extent=1.5)
    _check_pim(g, pts, filtered=True)
    ids, objs = api.compact_hits(torch.from_numpy(_pim(g, pts, filtered=True)[0]).cuda())
    want = bind.pim(g.vertices, g.indices, g.tri2obj, pts, filtered=True)
    assert np.array_equal(ids.cpu().numpy(), np.nonzero(want >= 0)[0])
    assert np.array_equal(objs.cpu().numpy(), want[want >= 0])


def test_pim_empty_and_tiny_meshes(cuda):
    pts = np.random.default_rng(0).uniform(-1, 1, size=(1000, 3)).astype(np.float32)
    V, F = synth.cube_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    one = synth.make_geometry(V, F[:1], np.zeros(1, np.int32), edges=False)
    _check_pim(one, pts)
    two = synth.make_geometry(V, F[:2], np.zeros(2, np.int32), edges=False)
    _check_pim(two, pts)
    cube = synth.make_geometry(V, F, np.zeros(12, np.int32), edges=False)
    _check_pim(cube, pts)
    empty = synth.make_geometry(V, F[:0], np.zeros(0, np.int32), edges=False)
    got, _ = _pim(empty, pts)
    assert (got == -1).all()


def _join(A, B, containment=False, cap=1 << 12, direction=0, pow2=True):
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ps = api.PairSet(cap, pow2=pow2)
    api.overlap_join(ba, bb, ps, direction=direction, with_containment=containment)
    return ps.finalize().cpu().numpy().astype(np.uint64), ps


def test_overlap_join_matches_oracle(cuda):
    A, B = synth.overlap_workload(n_objects=400, level=2, world=25.0, seed=1)
    got, _ = _join(A, B)
    want = bind.overlap_join(A, B)
    assert len(want) > 50
    assert np.array_equal(got, want)


def test_overlap_join_directions(cuda):
    A, B = synth.overlap_workload(n_objects=200, level=1, world=15.0, seed=6)
    got1, _ = _join(A, B, direction=1)
    got2, _ = _join(A, B, direction=2)
    w1 = bind.edge_join(A.edges, B.vertices, B.indices, B.tri2obj, swap=False)
    w2 = bind.edge_join(B.edges, A.vertices, A.indices, A.tri2obj, swap=True)
    assert np.array_equal(got1, w1) and np.array_equal(got2, w2)


def test_self_join_contains_diagonal(cuda):
    A, _ = synth.overlap_workload(n_objects=100, level=2, world=30.0, seed=2)
    got, _ = _join(A, A)
    assert np.array_equal(got, bind.overlap_join(A, A))
    pairs = api.keys_to_pairs(got)
    diag = set(int(i) for i, j in pairs if i == j)
    assert len(diag) >= 95  # nearly every object finds itself through a shared vertex


def test_overlap_table_growth(cuda):
    A, B = synth.overlap_workload(n_objects=600, level=1, world=15.0, seed=8)
    got, ps = _join(A, B, cap=1024)
    cap, _ = ps.info()
    want = bind.overlap_join(A, B)
    assert len(want) > 1024 and cap > 1024
    assert np.array_equal(got, want)


def test_intersection_join_with_containment(cuda):
    rng = np.random.default_rng(11)
    levels_a = rng.integers(1, 4, size=120)
    A = synth.mixed_level_set(120, levels_a, 0.5, 3.0, 30.0, rng)
    levels_b = rng.integers(1, 4, size=120)
    B = synth.mixed_level_set(120, levels_b, 0.2, 2.0, 30.0, rng, inside_of=(A._centers, A._radii),
                              inside_frac=0.2)
    got, _ = _join(A, B, containment=True, pow2=False, cap=rng.integers(1000, 3000) | 1)
    want = bind.intersection_join(A, B)
    assert np.array_equal(got, want)
    cont = bind.containment(B, A.vertices, A.indices, A.tri2obj, swap=True)
    ov = bind.overlap_join(A, B)
    assert len(np.setdiff1d(cont, ov)) >= 10  # pairs only the containment fallback finds


def test_mesh_overlap_order(cuda):
    A, B = synth.overlap_workload(n_objects=300, level=1, world=15.0, seed=12)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ps = api.PairSet(1 << 14)
    api.overlap_join(api.Bvh(da), api.Bvh(db), ps)
    k1 = ps.finalize(order=1).cpu().numpy().astype(np.uint64)
    pairs = api.keys_to_pairs(k1)
    # ascending by (id2, id1): MeshQueryResult{id1,id2} sorted as little-endian u64
    le = (pairs[:, 1].astype(np.uint64) << np.uint64(32)) | pairs[:, 0].astype(np.uint64)
    assert np.all(np.diff(le.astype(np.float64)) > 0) or len(le) < 2
    assert np.array_equal(np.sort(k1), bind.overlap_join(A, B))


def test_estimator_matches_oracle(cuda):
    A, B = synth.overlap_workload(n_objects=2000, level=1, world=100.0, seed=1, grid_resolution=32)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    est, raw = api.estimate_pairs(da, db)
    want_est, want_raw = bind.estimate_pairs(A.grid, B.grid)
    assert raw == pytest.approx(want_raw, rel=1e-5)
    assert abs(est - want_est) <= max(1, 1e-5 * want_est)
    # reference-compatible host entry point
    cv = api.cell_volume(A.grid)
    ca = np.ascontiguousarray(A.grid.cells)
    cb = np.ascontiguousarray(B.grid.cells)
    f = _lib.load().rs_estimate_overlap_selectivity(ca.ctypes.data, cb.ctypes.data, len(ca), cv, 0.001, 0.8)
    assert f == pytest.approx(want_raw, rel=1e-5)


def test_compact_hash_table_pairs_compat(cuda):
    rng = np.random.default_rng(2)
    table = np.full(5000, np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)
    pos = rng.choice(5000, size=700, replace=False)
    keys = (rng.integers(0, 1000, 700).astype(np.uint64) << np.uint64(32)) | rng.integers(0, 1000, 700).astype(np.uint64)
    table[pos] = keys
    d_t = torch.from_numpy(table.view(np.int64).copy()).cuda()
    out = torch.zeros(800, dtype=torch.int32, device="cuda").view(-1)
    out = torch.zeros(1600, dtype=torch.int32, device="cuda")
    n = _lib.load().compact_hash_table_pairs(d_t.data_ptr(), 5000, out.data_ptr(), 800)
    assert n == 700
    got = out.cpu().numpy().reshape(-1, 2)[:n]
    want_keys = table[np.sort(pos)]
    assert np.array_equal(got[:, 0].astype(np.uint64), want_keys >> np.uint64(32))
    assert np.array_equal(got[:, 1].astype(np.uint64), want_keys & np.uint64(0xffffffff))


def test_count_and_compact_hits_compat(cuda):
    rng = np.random.default_rng(3)
    n = 10_001
    rr = np.stack([np.arange(n), np.where(rng.uniform(size=n) < 0.3, rng.integers(0, 9, n), -1)], 1).astype(np.int32)
    d = torch.from_numpy(rr.copy()).cuda()
    L = _lib.load()
    assert L.count_hits_gpu(d.data_ptr(), n) == int((rr[:, 1] != -1).sum())
    out = torch.zeros_like(d)
    import ctypes
    h = ctypes.c_int()
    L.compact_hits_gpu(d.data_ptr(), out.data_ptr(), n, ctypes.byref(h))
    assert h.value == int((rr[:, 1] != -1).sum())
    assert np.array_equal(out.cpu().numpy()[: h.value], rr[rr[:, 1] != -1])


@pytest.mark.parametrize("leaf", [1, 3, 4, 8, 16])
def test_overlap_join_leaf_sizes(cuda, leaf):
    """Every leaf size builds a tree (groups of max(1, leaf / 2) triangles, leaves of up to
    `leaf`) whose traversal gives the oracle's pair set, with and without the broad phase;
    oblique point-in-mesh rays traverse the same tree."""
    A, B = synth.overlap_workload(n_objects=300, level=2, world=22.0, seed=4)
    want = bind.overlap_join(A, B)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da, leaf_size=leaf), api.Bvh(db, leaf_size=leaf)
    L = _lib.load()
    for cull in (1, 0):
        L.rs_set_overlap_cull(cull)
        ps = api.PairSet(1 << 14)
        api.overlap_join(ba, bb, ps)
        got = np.sort(ps.finalize().cpu().numpy().astype(np.uint64))
        np.testing.assert_array_equal(got, want)
    L.rs_set_overlap_cull(1)
    g, pts = synth.pim_workload(20_000, level=3, seed=5)
    d = np.array([0.3, -0.5, 0.81], np.float64)
    d = tuple(float(x) for x in (d / np.linalg.norm(d)).astype(np.float32))
    _check_pim(g, pts, direction=d, leaf=leaf)
    ba.close()
    bb.close()
