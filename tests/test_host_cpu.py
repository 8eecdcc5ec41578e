"""Host-side logic that needs no GPU: the bench's clock summary, the synthetic sets'
object layout (each object's triangles stored together, which the sharded join's
containment ranges rely on), and the invariant the edge payload's slab index relies on."""
import numpy as np

from rayspace3d_gb300 import synth


def test_synthetic_sets_store_objects_together():
    A, B = synth.overlap_workload(n_objects=50, level=2, world=100.0, seed=3)
    for g in (A, B):
        heads = np.flatnonzero(np.concatenate(([True], g.tri2obj[1:] != g.tri2obj[:-1])))
        assert len(heads) == 50 and np.all(np.diff(np.append(heads, len(g.tri2obj))) == 320)
        assert len(np.unique(g.tri2obj[heads])) == 50


def test_clock_summary(tmp_path, monkeypatch):
    import bench
    c = bench.Clocks(0)
    c.path = str(tmp_path / "clocks.csv")
    (tmp_path / "clocks.csv").write_text(
        "2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active\n"
        "1980, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active\n"
        "garbage line\n"
        "2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
    c.proc = object()  # a sampler that ran
    got = c.summary()
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3, "reasons": ["sw_power_cap"]}
    c.proc = None
    assert c.summary()["reasons"] == ["nvidia-smi unavailable"]


def _llround(y):
    """C's llround (halves away from zero) of float64 values (a - floor(a) is exact)."""
    a = np.abs(y)
    f = np.floor(a)
    return (np.sign(y) * np.where(a - f >= 0.5, f + 1.0, f)).astype(np.int64)


def _slab_cover(g, slab=256):
    """The slab index's invariant, restated on the host: with the payload's keys (the
    quantised x of each edge's lower endpoint) non-decreasing, the slabs an object's box
    selects by binary search over the slab keys hold every edge that has the object as a
    source."""
    e = g.edges
    q = lambda x: _llround(x.astype(np.float64) * 1e5)
    key = np.minimum(q(e.starts[:, 0]), q(e.ends[:, 0]))
    assert np.all(np.diff(key) >= 0), "payload not in the reference's key order"
    xq = key[::slab]
    n_obj = int(g.tri2obj.max()) + 1
    lo = np.full(n_obj, np.inf, np.float32)
    hi = np.full(n_obj, -np.inf, np.float32)
    vx = g.vertices[g.indices, 0]  # [nF, 3]
    np.minimum.at(lo, g.tri2obj, vx.min(axis=1))
    np.maximum.at(hi, g.tri2obj, vx.max(axis=1))
    first = np.maximum(np.searchsorted(xq, q(lo), side="left") - 1, 0)
    end = np.searchsorted(xq, q(hi), side="right")  # slabs [first, end)
    slab_of_edge = np.arange(len(key)) // slab
    for i in range(len(key)):
        for o in e.sources[e.offsets[i]:e.offsets[i] + e.counts[i]]:
            assert first[o] <= slab_of_edge[i] < end[o], (i, o)


def test_slab_index_covers_every_edge_of_its_objects():
    A, B = synth.overlap_workload(n_objects=120, level=2, world=40.0, seed=8)
    _slab_cover(A)
    _slab_cover(B, slab=16)
    # Shared edges (quantised-equal endpoints of touching cubes) carry several sources.
    g = synth.cube_grid(4, 3, 2)
    assert (g.edges.counts > 1).any()
    _slab_cover(g, slab=8)


def test_llround_matches_c():
    y = np.array([0.5, 1.5, 2.5, -0.5, -1.5, 0.49999999999999994, -0.49999999999999994, 2.4, -2.6, 1e10 + 0.5])
    assert _llround(y).tolist() == [1, 2, 3, -1, -2, 0, 0, 2, -3, 10000000001]
