"""Host-side logic that needs no GPU: the bench's clock summary, and the synthetic sets'
object layout (each object's triangles stored together, which the sharded join's
containment ranges rely on)."""
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
