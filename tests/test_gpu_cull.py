"""The overlap join's broad phase: the pair set is identical with culling on and off and
equal to the oracle's, on contact-heavy inputs (face-sharing and touching cubes, shared
edges, objects that only touch within the edge payload's quantisation) and on a query that
exhausts its node budget (one object whose box covers the whole other set)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, formats, synth

pytestmark = pytest.mark.gpu


def _join(A, B, cull, containment=False, indexed=False):
    L = _lib.load()
    L.rs_set_overlap_cull(1 if cull else 0)
    try:
        da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
        ba, bb = api.Bvh(da), api.Bvh(db)
        ps = api.PairSet(1 << 12)
        indexes = (api.edge_index(da)[0], api.edge_index(db)[0]) if indexed else None
        api.overlap_join(ba, bb, ps, with_containment=containment, indexes=indexes)
        torch.cuda.synchronize()
        return np.sort(ps.finalize().cpu().numpy().astype(np.uint64))
    finally:
        L.rs_set_overlap_cull(1)


def _check(A, B, containment=False):
    """The oracle's pair set from the join with the broad phase off, on, and on with the
    payloads' slab indexes."""
    want = bind.intersection_join(A, B) if containment else bind.overlap_join(A, B)
    on = _join(A, B, True, containment)
    off = _join(A, B, False, containment)
    slabs = _join(A, B, True, containment, indexed=True)
    np.testing.assert_array_equal(off, want)
    np.testing.assert_array_equal(on, want)
    np.testing.assert_array_equal(slabs, want)
    return want


def _shift(g, d, grid=False):
    V = (g.vertices + np.asarray(d, np.float32)).astype(np.float32)
    return synth.make_geometry(V, g.indices, g.tri2obj)


@pytest.mark.parametrize("offset", [(1.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.0, 0.0, 1.0), (1.0, 1.0, 1.0),
                                    (2.0, 0.0, 0.0), (3.0, 0.0, 0.0), (1e-5, 0.0, 0.0), (3.0 + 4e-6, 0.0, 0.0),
                                    (0.25, 0.0, 0.75)])
def test_cull_on_touching_cubes(cuda, offset):
    A = synth.cube_grid(3, 2, 2)
    B = _shift(synth.cube_grid(3, 2, 2), offset)
    _check(A, B)


def test_cull_on_random_spheres_and_intersection(cuda):
    for seed, world in [(21, 6.0), (22, 15.0), (23, 40.0)]:
        A, B = synth.overlap_workload(n_objects=200, level=1, world=world, seed=seed)
        _check(A, B)
    A, B = synth.overlap_workload(n_objects=150, level=1, world=10.0, seed=24)
    _check(A, B, containment=True)


def test_cull_with_shared_edges(cuda):
    """Edges shared by several objects (quantised-equal endpoints) carry the first
    object's endpoints; every source must still see its pairs."""
    g = synth.cube_grid(4, 1, 1)
    assert (g.edges.counts > 1).any()
    B = _shift(synth.cube_grid(2, 2, 2), (1.5, -0.5, 0.25))
    _check(g, B)
    _check(B, g)


@pytest.mark.parametrize("n_small", [3, 8, 9, 40])
def test_partner_lists_up_to_and_past_eight(cuda, n_small):
    """A sphere shell crossed by n small spheres on its surface: its query lists n partner
    objects (up to 8 listed, more marks all its edges live), and each small sphere has the
    shell as its one partner, so only its edges near the shell's box are traced.  The pairs
    equal the oracle's with the broad phase on and off."""
    rng = np.random.default_rng(100 + n_small)
    v, f = synth.icosphere(3)
    shell = synth.make_geometry((v * 5.0).astype(np.float32), f, np.zeros(len(f), np.int32))
    dirs = rng.normal(size=(n_small, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    vs, fs = synth.icosphere(2)
    Vs, Is, Ts = [], [], []
    for k in range(n_small):
        Vs.append((vs * 0.7 + dirs[k] * 5.0).astype(np.float32))
        Is.append(fs + np.uint32(len(vs) * k))
        Ts.append(np.full(len(fs), k, np.int32))
    small = synth.make_geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts))
    want = _check(shell, small)
    assert len(want) == n_small
    _check(small, shell)


def test_cull_budget_exhausted(cuda):
    """One huge sphere around a cloud of small ones: its query visits more nodes than the
    budget allows, which must switch culling off for the other side, not drop pairs."""
    rng = np.random.default_rng(5)
    small = synth.sphere_set(400, 2, 0.2, 0.6, 20.0, rng)
    v, f = synth.icosphere(3)
    big = synth.make_geometry((v * 9.0 + 10.0).astype(np.float32), f, np.zeros(len(f), np.int32))
    _check(big, small)
    _check(small, big)


def test_overlap_join_after_events_matches(cuda):
    """rs_overlap_join_after: the edge payloads are copied on another stream after the call
    is queued; each direction's rays wait for their event.  Same pair set as the plain join."""
    A, B = synth.overlap_workload(n_objects=300, level=2, world=30.0, seed=9)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ps = api.PairSet(1 << 14)
    api.overlap_join(ba, bb, ps)
    want = np.sort(ps.finalize().cpu().numpy())
    # fresh edge buffers written by a copy stream that first waits on a slow kernel
    host = [[t.cpu().pin_memory() for t in g.edges] for g in (da, db)]
    for g in (da, db):
        g.edges = tuple(torch.zeros_like(t) for t in g.edges)
    cs = torch.cuda.Stream()
    evs = [torch.cuda.Event(), torch.cuda.Event()]
    with torch.cuda.stream(cs):
        torch.cuda._sleep(20_000_000)  # keep the copies behind the join's queueing
        for k, g in enumerate((da, db)):
            for d, h in zip(g.edges, host[k]):
                d.copy_(h, non_blocking=True)
            evs[k].record(cs)
    ps2 = api.PairSet(1 << 14)
    api.overlap_join(ba, bb, ps2, edges_ready=(evs[0], evs[1]))
    got = np.sort(ps2.finalize().cpu().numpy())
    np.testing.assert_array_equal(got, want)
    assert len(got) > 0
    ba.close()
    bb.close()


@pytest.mark.parametrize("world,containment", [(30.0, False), (8.0, False), (400.0, False), (30.0, True)])
def test_filtered_join_matches_full_join(cuda, world, containment):
    """rs_overlap_join_filtered: BVHs over the objects whose boxes overlap the other set's
    only; the pair set equals the join over full BVHs (and the oracle's)."""
    A, B = synth.overlap_workload(n_objects=300, level=2, world=world, seed=12)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ps = api.PairSet(1 << 12)
    api.overlap_join(ba, bb, ps, with_containment=containment)
    want = np.sort(ps.finalize().cpu().numpy())
    for direction in (0, 1, 2):
        ps2 = api.PairSet(1 << 8)  # small: exercises the table growth
        api.overlap_join_filtered(da, db, ps2, direction=direction, with_containment=containment)
        got = np.sort(ps2.finalize().cpu().numpy())
        if direction == 0:
            np.testing.assert_array_equal(got, want)
        else:
            ps3 = api.PairSet(1 << 12)
            api.overlap_join(ba, bb, ps3, direction=direction, with_containment=containment)
            np.testing.assert_array_equal(got, np.sort(ps3.finalize().cpu().numpy()))
    if not containment and world == 30.0:
        np.testing.assert_array_equal(want.astype(np.uint64), bind.overlap_join(A, B))
    ba.close()
    bb.close()


def test_filtered_join_with_an_empty_set(cuda):
    A, _ = synth.overlap_workload(n_objects=50, level=1, world=10.0, seed=2)
    V, F = synth.cube_mesh((0, 0, 0), (1, 1, 1))
    empty = synth.make_geometry(V, F[:0], np.zeros(0, np.int32), edges=False)
    da, de = api.DeviceGeometry(A), api.DeviceGeometry(empty)
    de.edges = (torch.zeros((0, 3), device="cuda"), torch.zeros((0, 3), device="cuda")) + tuple(
        torch.zeros(0, dtype=torch.int32, device="cuda") for _ in range(3))
    ps = api.PairSet(1 << 8)
    api.overlap_join_filtered(da, de, ps, with_containment=True)
    assert ps.finalize().numel() == 0


def test_cull_with_sparse_object_ids(cuda):
    """Object ids far above the triangle count: the build's object boxes do not cover them,
    so the broad phase computes the boxes itself; the pairs stay the oracle's."""
    A, B = synth.overlap_workload(n_objects=150, level=1, world=10.0, seed=31)
    A2 = synth.make_geometry(A.vertices, A.indices, A.tri2obj * 4001 + 3)
    B2 = synth.make_geometry(B.vertices, B.indices, B.tri2obj * 7 + 1)
    assert int(A2.tri2obj.max()) + 1 > len(A2.indices)
    _check(A2, B2)
    _check(B2, A2, containment=True)


@pytest.mark.parametrize("n_objects, world", [(150, 10.0), (2500, 12.0)])
def test_finalize_orders_and_count(cuda, n_objects, world):
    """Both finalize paths (gather + one-block sort up to 4096 keys, radix sort above): the
    keys ascending as (id1, id2) for order 0 and as (id2, id1) for order 1, the count from the
    join's own status read, and the same result on a second call."""
    A, B = synth.overlap_workload(n_objects=n_objects, level=1, world=world, seed=32)
    want = bind.overlap_join(A, B)
    ps = api.PairSet(1 << 16)
    api.overlap_join(api.Bvh(api.DeviceGeometry(A)), api.Bvh(api.DeviceGeometry(B)), ps)
    assert ps.info()[1] == len(want)
    k0 = ps.finalize(order=0).cpu().numpy().astype(np.uint64)
    np.testing.assert_array_equal(k0, want)
    k1 = ps.finalize(order=1).cpu().numpy().astype(np.uint64)
    swapped = (k1 << np.uint64(32)) | (k1 >> np.uint64(32))
    assert np.all(swapped[1:] > swapped[:-1])
    np.testing.assert_array_equal(np.sort(k1), want)
    np.testing.assert_array_equal(ps.finalize(order=0).cpu().numpy().astype(np.uint64), want)
    # through the C ABI with the default wait, and with too small an output buffer
    L = _lib.load()
    out = torch.empty(max(len(want), 1), dtype=torch.int64, device="cuda")
    n = ctypes.c_uint64()
    assert L.rs_pairset_finalize(ps.handle, 0, out.data_ptr(), len(want), ctypes.byref(n), None) == 0
    assert n.value == len(want)
    np.testing.assert_array_equal(out[:n.value].cpu().numpy().astype(np.uint64), want)
    if len(want) > 1:
        rc = L.rs_pairset_finalize(ps.handle, 0, out.data_ptr(), len(want) - 1, ctypes.byref(n), None)
        assert rc == _lib.RS_ERR_OUTPUT_OVERFLOW and n.value == len(want)
    assert (len(want) <= 4096) == (n_objects == 150)
    ps.clear()
    assert ps.info()[1] == 0
    assert ps.finalize().numel() == 0


def test_overlap_join_reads_pinned_host_payloads(cuda):
    """Edge payloads left in pinned host memory (the endpoints only, then all five arrays) are
    read in place through their mapped addresses: the same pair set as device payloads.
    rs_kernel_pointer maps pinned memory and refuses pageable memory (checked without a
    launch: no kernel is ever given a pageable address)."""
    A, B = synth.overlap_workload(n_objects=300, level=2, world=30.0, seed=9)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ps = api.PairSet(1 << 14)
    api.overlap_join(ba, bb, ps)
    want = np.sort(ps.finalize().cpu().numpy())
    assert len(want) > 0
    device = [g.edges for g in (da, db)]
    for k_host in (2, 5):
        for g, e in zip((da, db), device):
            g.edges = tuple(t.cpu().pin_memory() if k < k_host else t for k, t in enumerate(e))
        ps2 = api.PairSet(1 << 14)
        api.overlap_join(ba, bb, ps2)
        np.testing.assert_array_equal(np.sort(ps2.finalize().cpu().numpy()), want)
    L = _lib.load()
    out = ctypes.c_void_p()
    pinned = torch.zeros(16, dtype=torch.float32).pin_memory()
    assert L.rs_kernel_pointer(pinned.data_ptr(), ctypes.byref(out)) == 0 and out.value
    dev = torch.zeros(16, device="cuda")
    assert L.rs_kernel_pointer(dev.data_ptr(), ctypes.byref(out)) == 0 and out.value == dev.data_ptr()
    pageable = np.zeros(16, np.float32)
    assert L.rs_kernel_pointer(pageable.ctypes.data, ctypes.byref(out)) == _lib.RS_ERR_INVALID
    ba.close()
    bb.close()


def _key_x(v):
    return np.array([int(np.round(np.float64(x) * 1e5)) if abs(np.float64(x) * 1e5 - np.trunc(np.float64(x) * 1e5)) != 0.5
                     else int(np.trunc(np.float64(x) * 1e5) + np.sign(x)) for x in v], dtype=np.int64)


@pytest.mark.parametrize("world", [6.0, 30.0, 400.0])
def test_slab_index_and_indexed_join(cuda, world):
    """rs_edge_index's keys are the quantised x of each slab's first edge's lower endpoint
    (llround, halves away from zero); the indexed join equals the oracle with the payloads on
    the device and with payloads and indexes in pinned host memory, in both directions and
    with one index missing.  A shuffled payload is reported out of order, and the join with
    its index (which then covers every slab) is still exact."""
    A, B = synth.overlap_workload(n_objects=300, level=2, world=world, seed=33)
    want = bind.overlap_join(A, B)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ia, oka = api.edge_index(da)
    ib, okb = api.edge_index(db)
    assert oka and okb
    e = A.edges
    first = np.arange(0, len(e.starts), 256)
    keys = np.minimum(_key_x(e.starts[first, 0]), _key_x(e.ends[first, 0]))
    got = ia.cpu().numpy()
    assert got[0] == 1 and got[1] == int(e.sources.max()) and got[2] == len(e.starts)
    np.testing.assert_array_equal(got[3:], keys)

    def run(indexes, direction=0):
        ps = api.PairSet(1 << 12)
        api.overlap_join(ba, bb, ps, direction=direction, indexes=indexes)
        return np.sort(ps.finalize().cpu().numpy().astype(np.uint64))

    np.testing.assert_array_equal(run((ia, ib)), want)
    np.testing.assert_array_equal(run((ia, None)), want)
    for d in (1, 2):
        np.testing.assert_array_equal(run((ia, ib), d), run(None, d))
    # Payloads and indexes in pinned host memory, read in place.
    device = [g.edges for g in (da, db)]
    for g, ed in zip((da, db), device):
        g.edges = tuple(t.cpu().pin_memory() for t in ed)
    np.testing.assert_array_equal(run((ia.cpu().pin_memory(), ib.cpu().pin_memory())), want)
    for g, ed in zip((da, db), device):
        g.edges = ed
    # A payload out of key order.
    perm = np.random.default_rng(1).permutation(len(e.starts))
    shuffled = formats.Edges(e.starts[perm], e.ends[perm], e.offsets[perm], e.counts[perm], e.sources)
    A2 = synth.make_geometry(A.vertices, A.indices, A.tri2obj, edges=False)
    A2.edges = shuffled
    d2 = api.DeviceGeometry(A2)
    i2, ok2 = api.edge_index(d2)
    assert not ok2 and int(i2[0]) == 0
    b2 = api.Bvh(d2)
    ps = api.PairSet(1 << 12)
    api.overlap_join(b2, bb, ps, indexes=(i2, ib))
    np.testing.assert_array_equal(np.sort(ps.finalize().cpu().numpy().astype(np.uint64)), want)
    for h in (ba, bb, b2):
        h.close()
