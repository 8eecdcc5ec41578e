"""The N>1 host path of bench.py on CPU: two gloo ranks, each with its own join time,
combine to the slowest rank's step time and whole-job seconds per join (independent
joins per rank, no data-path collective)."""
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
