"""The clustered BVH build (rs_bvh_build_clustered): one tree per run of an object's
triangles, joined by a tree over the cluster boxes.  Its queries must give the oracle's
results exactly like the build over all triangles, for any partition of the triangles into
clusters of 1..512 (object runs, runs split across objects, a single cluster, single
triangles), every leaf size, and the build must refuse cluster starts that are not such a
partition."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu


def _bvh(dg, starts=None, leaf=0):
    """BVH of dg built per cluster with the given starts (default: the object runs)."""
    if starts is None:
        return 0, api.Bvh(dg, leaf_size=leaf, clustered=True)
    cs = torch.from_numpy(np.asarray(starts, np.uint32).view(np.int32)).cuda()
    h = ctypes.c_void_p()
    rc = _lib.load().rs_bvh_build_clustered(dg.V.data_ptr(), dg.nV, dg.I.data_ptr(), dg.nF, dg.T.data_ptr(),
                                            cs.data_ptr(), len(starts) - 1, leaf, 0, ctypes.byref(h), None)
    if rc:
        return rc, None
    b = api.Bvh.__new__(api.Bvh)
    b.geom, b.handle, b.clustered, b._starts = dg, h, True, cs
    return 0, b


def _join(ba, bb, containment=False):
    ps = api.PairSet(1 << 14)
    api.overlap_join(ba, bb, ps, with_containment=containment)
    return np.sort(ps.finalize().cpu().numpy().astype(np.uint64))


def _pim(bvh, pts):
    obj, inside = api.point_in_mesh(bvh, torch.from_numpy(np.ascontiguousarray(pts)).cuda())
    torch.cuda.synchronize()
    return obj.cpu().numpy()


@pytest.mark.parametrize("level, world, seed", [(1, 8.0, 41), (2, 20.0, 42), (2, 60.0, 43)])
def test_clustered_joins_match_oracle(cuda, level, world, seed):
    A, B = synth.overlap_workload(n_objects=300, level=level, world=world, seed=seed)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    assert da.clusters is not None and db.clusters is not None
    want = bind.overlap_join(A, B)
    want_int = bind.intersection_join(A, B)
    for clustered in (True, False):
        ba = api.Bvh(da, clustered=clustered)
        bb = api.Bvh(db, clustered=clustered)
        assert ba.clustered == clustered
        np.testing.assert_array_equal(_join(ba, bb), want)
        np.testing.assert_array_equal(_join(ba, bb, containment=True), want_int)


def test_clustered_pim_and_node_count(cuda):
    rng = np.random.default_rng(44)
    g = synth.sphere_set(60, 2, 0.5, 1.5, 6.0, rng, edges=False)
    pts = rng.uniform(-0.5, 6.5, size=(40_000, 3)).astype(np.float32)
    want = bind.pim(g.vertices, g.indices, g.tri2obj, pts)
    dg = api.DeviceGeometry(g)
    for leaf in (1, 2, 5, 16):
        rc, b = _bvh(dg, leaf=leaf)
        assert rc == 0
        np.testing.assert_array_equal(_pim(b, pts), want)
        assert b.info()["nodes"] == 60 - 1 + len(g.indices)
        b.close()


@pytest.mark.parametrize("kind", ["chunks100", "single", "ones", "mixed"])
def test_clustered_any_partition(cuda, kind):
    """Clusters need not follow objects: fixed chunks across object boundaries, one cluster
    for a whole small set, one triangle per cluster, and irregular sizes."""
    rng = np.random.default_rng(45)
    A = synth.sphere_set(6 if kind == "single" else 80, 1, 0.5, 1.5, 5.0, rng)
    B = synth.sphere_set(80, 1, 0.5, 1.5, 5.0, rng)
    n = len(A.indices)
    if kind == "chunks100":
        starts = list(range(0, n, 100)) + [n]
    elif kind == "single":
        assert n <= 512
        starts = [0, n]
    elif kind == "ones":
        starts = list(range(n + 1))
    else:
        cuts = np.sort(rng.choice(np.arange(1, n), size=n // 37, replace=False))
        starts = [0] + cuts.tolist() + [n]
        assert int(np.diff(starts).max()) <= 512
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    rc, ba = _bvh(da, starts)
    assert rc == 0
    bb = api.Bvh(db)
    np.testing.assert_array_equal(_join(ba, bb, containment=True), bind.intersection_join(A, B))
    np.testing.assert_array_equal(_join(bb, ba), bind.overlap_join(B, A))
    pts = rng.uniform(-0.5, 5.5, size=(20_000, 3)).astype(np.float32)
    np.testing.assert_array_equal(_pim(ba, pts), bind.pim(A.vertices, A.indices, A.tri2obj, pts))


def test_clustered_tiny_sets(cuda):
    V, F = synth.cube_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    pts = np.random.default_rng(46).uniform(-1, 1, size=(2000, 3)).astype(np.float32)
    for m in (1, 2, 3, 12):
        g = synth.make_geometry(V, F[:m], np.zeros(m, np.int32), edges=False)
        for leaf in (1, 2, 16):
            rc, b = _bvh(api.DeviceGeometry(g), leaf=leaf)
            assert rc == 0
            np.testing.assert_array_equal(_pim(b, pts), bind.pim(g.vertices, g.indices, g.tri2obj, pts))


def test_clustered_rejects_bad_starts(cuda):
    v, f = synth.icosphere(3)  # 1280 triangles: one object too large for one cluster
    g = synth.make_geometry(v.astype(np.float32), f, np.zeros(len(f), np.int32), edges=False)
    dg = api.DeviceGeometry(g)
    assert dg.clusters is None
    with pytest.raises(ValueError):
        api.Bvh(dg, clustered=True)
    n = len(f)
    bad = [[0, n],                      # a cluster over 512
           [0, 100, 100, n],            # an empty cluster
           [0, 300, 200, n],            # decreasing
           [5, 300, 600, 900, n],       # not starting at 0
           [0, 300, 600, 900, n - 1],   # not ending at nF
           [0, 300, 600, 900, n + 1]]   # past nF
    for starts in bad:
        rc, _ = _bvh(dg, starts)
        assert rc == _lib.RS_ERR_INVALID, starts
    ok = [0, 300, 600, 900, n]
    rc, b = _bvh(dg, ok)
    assert rc == 0
    pts = np.random.default_rng(47).uniform(-1.5, 1.5, size=(5000, 3)).astype(np.float32)
    np.testing.assert_array_equal(_pim(b, pts), bind.pim(g.vertices, g.indices, g.tri2obj, pts))
    # host-side checks: no clusters for a non-empty set, more clusters than triangles
    h = ctypes.c_void_p()
    L = _lib.load()
    cs = torch.zeros(2, dtype=torch.int32, device="cuda")
    assert L.rs_bvh_build_clustered(dg.V.data_ptr(), dg.nV, dg.I.data_ptr(), dg.nF, dg.T.data_ptr(), cs.data_ptr(),
                                    0, 0, 0, ctypes.byref(h), None) == _lib.RS_ERR_INVALID
    assert L.rs_bvh_build_clustered(dg.V.data_ptr(), dg.nV, dg.I.data_ptr(), dg.nF, dg.T.data_ptr(), cs.data_ptr(),
                                    n + 1, 0, 0, ctypes.byref(h), None) == _lib.RS_ERR_INVALID
