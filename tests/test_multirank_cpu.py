"""The N>1 host paths on CPU gloo ranks: bench.py's rank combination, and the sharded
join and point-in-mesh of rayspace3d_gb300/shard.py, whose merged results must equal the
single-rank oracle's."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        res = {"ms_per_step": 1.0 + rank, "value": (1.0 + rank) / 1e3, "e2e": {"value": 0.003 * (1 + rank)}}
        bench.combine_ranks(res, world, "cpu")
        out[rank] = (res["ms_per_step"], res["value"], res["e2e"]["value"])
    finally:
        dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        got = dict(out)
    # slowest rank: 2 ms per step; 2 joins in it -> 1 ms per join; e2e 6 ms -> 3 ms per join
    for r in range(2):
        assert got[r][0] == pytest.approx(2.0)
        assert got[r][1] == pytest.approx(0.001)
        assert got[r][2] == pytest.approx(0.003)


def test_reference_arm_other_ranks_exit_without_work(tmp_path):
    """--impl reference under torchrun: ranks > 0 return at once (exit 0, no output)."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    # rank 1 alone: the CPU arm joins no process group, so it neither waits for rank 0 nor works
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


# --- the sharded join and point-in-mesh (rayspace3d_gb300/shard.py) on gloo ranks ------
#
# Each rank computes its share with the oracle on the same slices the engine path hands
# to the GPU (edge ranges of both payloads, containment object ranges cut at object
# boundaries, point ranges); the exchange is shard.gather_keys / shard.gather_ranges.

def _shard_case():
    from rayspace3d_gb300 import synth
    A, B = synth.overlap_workload(n_objects=200, level=1, world=12.0, seed=3)
    g, pts = synth.pim_workload(20_000, level=2, seed=1)
    return A, B, g, pts


def _shard_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import numpy as np
        from oracle import bind
        from rayspace3d_gb300 import shard
        from rayspace3d_gb300.formats import Edges, Geometry
        A, B, g, pts = _shard_case()
        keys = []
        for src, tgt, swap in ((A, B, False), (B, A, True)):
            lo, hi = shard.split_range(len(src.edges.starts), world, rank)
            e = src.edges
            part = Edges(*shard.slice_edges((e.starts, e.ends, e.offsets, e.counts, e.sources), lo, hi))
            keys.append(bind.edge_join(part, tgt.vertices, tgt.indices, tgt.tri2obj, swap=swap))
            cuts = shard.object_cuts(src.tri2obj, world)
            tlo, thi = cuts[rank]
            if thi > tlo:
                sub = Geometry(src.vertices, src.indices[tlo:thi], src.tri2obj[tlo:thi])
                keys.append(bind.containment(sub, tgt.vertices, tgt.indices, tgt.tri2obj, swap=swap))
        local = np.unique(np.concatenate(keys)).astype(np.uint64)
        merged = shard.gather_keys(torch.from_numpy(local.view(np.int64)))
        lo, hi = shard.split_range(len(pts), world, rank)
        obj = torch.from_numpy(bind.pim(g.vertices, g.indices, g.tri2obj, pts[lo:hi]))
        allobj = shard.gather_ranges(obj, len(pts), rank, world)
        out[rank] = (merged.numpy().view(np.uint64).tolist(), len(local), allobj.numpy().tolist())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_join_equals_single_rank(world):
    import numpy as np
    from oracle import bind
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_shard_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        got = dict(out)
    A, B, g, pts = _shard_case()
    want = bind.intersection_join(A, B)
    want_obj = bind.pim(g.vertices, g.indices, g.tri2obj, pts)
    assert len(want) > 50
    for r in range(world):
        np.testing.assert_array_equal(np.array(got[r][0], np.uint64), want)
        assert got[r][1] < len(want)  # every rank held only part of the pairs
        np.testing.assert_array_equal(np.array(got[r][2], np.int32), want_obj)


def test_object_cuts():
    import numpy as np
    from rayspace3d_gb300 import shard
    t = np.repeat(np.arange(10), [3, 1, 4, 1, 5, 9, 2, 6, 5, 3])
    cuts = shard.object_cuts(t, 3)
    assert cuts[0][0] == 0 and cuts[-1][1] == len(t)
    for (a, b), (c, d) in zip(cuts, cuts[1:]):
        assert b == c and (b == len(t) or t[b] != t[b - 1])
    assert shard.object_cuts(np.array([0, 0, 1, 0]), 2) is None  # object 0 in two runs
    assert [shard.split_range(10, 3, r) for r in range(3)] == [(0, 4), (4, 7), (7, 10)]
