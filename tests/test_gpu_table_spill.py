"""Pair-table growth through the overflow table: once a table far smaller than the join's pair
count passes 3/4 load, later keys that do not settle at their first slot go to the pair set's
overflow table, and the join's status read regrows the table from both instead of rerunning the
rays.  The pair set equals the oracle's, and the launch count shows that no ray launch ran
twice."""
import ctypes

import numpy as np
import pytest
import torch

import edge_cases as ec
from oracle import bind
from rayspace3d_gb300 import _lib, api, synth
from rayspace3d_gb300.formats import Geometry

pytestmark = pytest.mark.gpu


def _launches(fn):
    L = _lib.load()
    torch.cuda.synchronize()
    n0 = L.rs_launch_count()
    fn()
    torch.cuda.synchronize()
    return L.rs_launch_count() - n0


@pytest.mark.parametrize("containment", [False, True])
def test_overlap_join_regrows_from_the_overflow_table(cuda, containment):
    A, B = synth.overlap_workload(n_objects=300, level=2, world=12.0, seed=41)
    want = bind.intersection_join(A, B) if containment else bind.overlap_join(A, B)
    assert len(want) > 256
    ba, bb = api.Bvh(api.DeviceGeometry(A)), api.Bvh(api.DeviceGeometry(B))
    big = api.PairSet(1 << 16)
    api.overlap_join(ba, bb, big, with_containment=containment)  # first use: lazily built state
    big.clear()
    n_big = _launches(lambda: api.overlap_join(ba, bb, big, with_containment=containment))
    small = api.PairSet(16)
    n_small = _launches(lambda: api.overlap_join(ba, bb, small, with_containment=containment))
    for ps in (big, small):
        np.testing.assert_array_equal(ps.finalize().cpu().numpy().astype(np.uint64), want)
    cap, count = small.info()
    assert count == len(want) and cap >= 2 * len(want)
    # The extra launches are the rehash of each regrowth, not a second pass of the rays.
    assert 1 <= n_small - n_big <= 8, (n_small, n_big)
    # A second join into the grown table needs no growth.
    small.clear()
    assert _launches(lambda: api.overlap_join(ba, bb, small, with_containment=containment)) == n_big
    np.testing.assert_array_equal(small.finalize().cpu().numpy().astype(np.uint64), want)
    ba.close()
    bb.close()


def test_edge_join_spills_with_the_odd_table(cuda):
    A, B, segs = ec.slab_stack()
    bb = api.Bvh(api.DeviceGeometry(B))
    src = api.DeviceGeometry(Geometry(A.vertices, A.indices, A.tri2obj, total_triangles=len(A.indices), edges=segs))
    want = bind.edge_join(segs, B.vertices, B.indices, B.tri2obj)
    assert len(want) > 16
    ps = api.PairSet(5, pow2=False)
    api.edge_join(bb, src, ps)
    np.testing.assert_array_equal(ps.finalize().cpu().numpy().astype(np.uint64), want)
    assert ps.info()[0] % 2 == 1


def test_batch_regrows_and_recaptures(cuda):
    """A batched edge join into a 4-slot table: rs_batch_wait regrows the spilled table, and
    the next submit recaptures its graph with the new slots."""
    L = _lib.load()
    A, B, segs = ec.slab_stack()
    bb = api.Bvh(api.DeviceGeometry(B))
    src = api.DeviceGeometry(Geometry(A.vertices, A.indices, A.tri2obj, total_triangles=len(A.indices), edges=segs))
    want = bind.edge_join(segs, B.vertices, B.indices, B.tri2obj)
    ps = api.PairSet(4)
    h = ctypes.c_void_p()
    assert L.rs_batch_create(ctypes.byref(h)) == 0
    try:
        assert L.rs_batch_add_edges(h, bb.handle, *src.edge_ptrs(), src.nE, 0, ps.handle, None) == 0
        s = torch.cuda.current_stream()
        caps = []
        for _ in range(3):
            ps.clear()
            assert L.rs_batch_submit(h, ctypes.c_void_p(s.cuda_stream)) == 0
            st = (ctypes.c_int * 1)()
            assert L.rs_batch_wait(h, st) == 0 and st[0] == 0
            np.testing.assert_array_equal(ps.finalize().cpu().numpy().astype(np.uint64), want)
            caps.append(ps.info()[0])
        assert caps[0] > 4 and caps[1] == caps[0] == caps[2]
    finally:
        L.rs_batch_destroy(h)
