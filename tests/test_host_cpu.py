"""Host-side logic that needs no GPU: the cluster starts of the clustered BVH build, the
bench's clock summary, and the synthetic sets' object layout the clustered build relies on."""
import numpy as np
import pytest

from rayspace3d_gb300 import api, synth


@pytest.mark.parametrize("ids, want", [
    ([0], [0, 1]),
    ([0, 0, 1, 1, 1, 2], [0, 2, 5, 6]),
    ([5, 5, 3, 3, 9], [0, 2, 4, 5]),          # runs need not be sorted by id
    ([1, 2, 1, 2], [0, 1, 2, 3, 4]),          # an object split into runs: each run a cluster
    ([-1, -1, 7], [0, 2, 3]),                 # negative ids are ids like any other
])
def test_cluster_starts_runs(ids, want):
    got = api.cluster_starts(np.asarray(ids, np.int32))
    assert got.dtype == np.uint32
    np.testing.assert_array_equal(got, want)


def test_cluster_starts_limits():
    assert api.cluster_starts(np.zeros(0, np.int32)) is None
    assert api.cluster_starts(np.zeros(api.MAX_CLUSTER, np.int32)) is not None
    assert api.cluster_starts(np.zeros(api.MAX_CLUSTER + 1, np.int32)) is None
    ids = np.repeat(np.arange(3, dtype=np.int32), [10, api.MAX_CLUSTER + 1, 10])
    assert api.cluster_starts(ids) is None
    assert len(api.cluster_starts(ids, max_size=1024)) == 4


def test_synthetic_sets_store_objects_together():
    A, B = synth.overlap_workload(n_objects=50, level=2, world=100.0, seed=3)
    for g in (A, B):
        cs = api.cluster_starts(g.tri2obj)
        assert cs is not None and len(cs) == 51
        assert np.all(np.diff(cs) == 320)


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


def test_device_geometry_clusters_on_first_use():
    """The cluster starts are computed from the host object ids when first asked for, can be
    overridden (a copy that builds over all triangles), and are absent for wrapped tensors
    and for objects over 512 triangles (on the CPU device: no GPU needed)."""
    import torch
    A, _ = synth.overlap_workload(n_objects=20, level=1, world=50.0, seed=2)
    g = api.DeviceGeometry(A, device="cpu")
    assert "_clusters" not in g.__dict__
    cs = g.clusters
    assert cs.dtype == torch.int32 and int(cs[-1]) == len(A.indices) and cs.shape[0] == 21
    copy = api.DeviceGeometry.__new__(api.DeviceGeometry)
    copy.__dict__.update(g.__dict__)
    copy.clusters = None
    assert copy.clusters is None and g.clusters is cs
    assert api.DeviceGeometry.from_tensors(g.V, g.I, g.T).clusters is None
    v, f = synth.icosphere(3)
    big = synth.make_geometry(v.astype(np.float32), f, np.zeros(len(f), np.int32), edges=False)
    assert api.DeviceGeometry(big, device="cpu").clusters is None
