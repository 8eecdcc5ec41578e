"""Legacy per-triangle overlap (rs_triangle_join, mesh_overlap.cu:126-179) against the
oracle's edge-ray join run on the per-triangle edge payload (each triangle's own edges in
its own orientation, the triangle's object as the one source).  Exact pair-key equality."""
import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, formats, synth

pytestmark = pytest.mark.gpu


def triangle_payload(g):
    """The per-triangle edges as an edge payload (the oracle's input)."""
    I = np.asarray(g.indices, np.int64)
    a = I[:, [0, 1, 2]].reshape(-1)
    b = I[:, [1, 2, 0]].reshape(-1)
    n = len(a)
    return formats.Edges(g.vertices[a], g.vertices[b], np.arange(n, dtype=np.int32), np.ones(n, np.int32),
                         np.repeat(np.asarray(g.tri2obj, np.int32), 3))


def _gpu(target, source, swap):
    bt, ds = api.Bvh(api.DeviceGeometry(target)), api.DeviceGeometry(source)
    ps = api.PairSet(1 << 16)
    api.triangle_join(bt, ds, ps, swap=swap)
    keys = np.sort(ps.finalize().cpu().numpy().astype(np.uint64))
    bt.close()
    return keys


@pytest.mark.parametrize("swap", [False, True])
def test_triangle_join_matches_oracle(cuda, swap):
    A, B = synth.overlap_workload(n_objects=400, level=2, world=40.0, seed=3)
    want = bind.edge_join(triangle_payload(A), B.vertices, B.indices, B.tri2obj, swap=swap)
    got = _gpu(B, A, swap)
    np.testing.assert_array_equal(got, want)
    assert len(got) > 100


def test_triangle_join_on_shared_vertices_and_grid_coincidences(cuda):
    """Cube grids whose faces and edges coincide with the other set's: the triangle edges
    run along the other mesh's edges and through its vertices."""
    A = synth.cube_grid(3, 3, 2)
    B = synth.cube_grid(2, 3, 3)
    B.vertices = (B.vertices + np.float32(0.5)).astype(np.float32)
    for swap in (False, True):
        want = bind.edge_join(triangle_payload(A), B.vertices, B.indices, B.tri2obj, swap=swap)
        np.testing.assert_array_equal(_gpu(B, A, swap), want)


def test_triangle_join_rejects_out_of_range_index(cuda):
    A, B = synth.overlap_workload(n_objects=20, level=1, world=5.0, seed=1)
    I = A.indices.copy()
    I[3, 1] = len(A.vertices) + 7
    bad = formats.Geometry(A.vertices, I, A.tri2obj, total_triangles=len(I))
    bt, ds = api.Bvh(api.DeviceGeometry(B)), api.DeviceGeometry(bad)
    ps = api.PairSet(1 << 12)
    st = _lib.load().rs_triangle_join(bt.handle, ds.V.data_ptr(), ds.nV, ds.I.data_ptr(), ds.nF, ds.T.data_ptr(), 0,
                                      ps.handle, None)
    assert st == 2  # RS_ERR_INVALID
    bt.close()
