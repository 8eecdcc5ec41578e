"""The query path split across ranks, one GPU per rank.

The reference runs on one device (query/src/optix/OptixContext.cpp:4-8).  Its join
shards with a single exchange step:

* the overlap join: each rank traces a contiguous range of A's edges against B and of B's
  edges against A (both BVHs built whole on every rank), and the containment rays of a
  contiguous range of each set's objects; it deduplicates its own pairs (the engine's pair
  table, sorted and unique on finalisation), then the ranks all-gather their sorted key
  runs and merge them;
* point-in-mesh: each rank answers a contiguous range of the points; the results are
  concatenated in rank order.

Edge ranges come from slicing the .pre edge payload: starts/ends/offsets/counts are cut,
the sources array is kept whole (offsets index it).  Containment ranges cut the triangle
arrays at object boundaries, which needs each object's triangles to be stored together (as
preprocess_dataset writes them); otherwise rank 0 runs every containment ray.

The exchange uses torch.distributed, so it runs over NCCL between GPUs and over gloo on
CPU ranks (which is how the host logic is tested).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch


def split_range(n: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous [lo, hi) share of n items for `rank` (sizes differ by at most one)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def object_cuts(tri2obj: np.ndarray, world: int) -> Optional[List[Tuple[int, int]]]:
    """Triangle ranges, one per rank, cut at object boundaries and balanced by triangle
    count; None when some object's triangles are not stored together."""
    t = np.asarray(tri2obj)
    n = len(t)
    if n == 0:
        return [(0, 0)] * world
    change = np.nonzero(t[1:] != t[:-1])[0] + 1
    starts = np.concatenate([[0], change])
    if len(np.unique(t[starts])) != len(starts):
        return None  # an object appears in two runs
    cuts = [0]
    for r in range(1, world):
        want = (n * r) // world
        k = int(np.searchsorted(starts, want))
        cuts.append(max(cuts[-1], int(starts[k]) if k < len(starts) else n))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def slice_edges(edges: Sequence, lo: int, hi: int):
    """The payload (starts, ends, offsets, counts, sources) of edges [lo, hi)."""
    s, e, off, cnt, src = edges
    return s[lo:hi], e[lo:hi], off[lo:hi], cnt[lo:hi], src


def gather_keys(local: torch.Tensor, group=None) -> torch.Tensor:
    """All-gather of every rank's sorted unique pair keys (int64 bit patterns of the u64
    keys id1 << 32 | id2, object ids below 2^31) and their merge: one sorted unique run.
    Runs of unequal length are padded to the longest and trimmed after the gather."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    n = torch.tensor([local.numel()], dtype=torch.int64, device=local.device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    sizes = [int(x.item()) for x in sizes]
    m = max(max(sizes), 1)
    padded = torch.full((m,), -1, dtype=torch.int64, device=local.device)
    padded[:local.numel()] = local
    runs = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(runs, padded, group=group)
    return merge_runs([r[:k] for r, k in zip(runs, sizes)])


def merge_runs(runs: Sequence[torch.Tensor]) -> torch.Tensor:
    """Merge of sorted runs into one sorted run without duplicates."""
    if not runs:
        return torch.zeros(0, dtype=torch.int64)
    cat = torch.cat(list(runs))
    if cat.numel() == 0:
        return cat
    return torch.unique_consecutive(torch.sort(cat).values)


def sharded_overlap_join(A, B, rank: int, world: int, with_containment: bool = False, group=None,
                         stream=None) -> torch.Tensor:
    """The join of two DeviceGeometry sets split across the ranks of `group`: this rank's
    edge ranges (and containment object ranges) through the engine, then the exchange.
    Every rank returns the whole sorted pair list (int64 keys on the GPU)."""
    from . import api
    ba, bb = api.Bvh(A, stream=stream), api.Bvh(B, stream=stream)
    la, ha = split_range(A.nE, world, rank)
    lb, hb = split_range(B.nE, world, rank)
    ea = slice_edges(A.edges, la, ha)
    eb = slice_edges(B.edges, lb, hb)
    ps = api.PairSet(1 << 16, stream=stream)
    api.overlap_join_edges(ba, ea, bb, eb, ps, stream=stream)
    if with_containment:
        for src, tgt, swap in ((A, bb, False), (B, ba, True)):
            cuts = object_cuts(src.host_tri2obj(), world)
            lo, hi = cuts[rank] if cuts is not None else ((0, src.nF) if rank == 0 else (0, 0))
            if hi > lo:
                api.containment_range(tgt, src, lo, hi, ps, swap=swap, stream=stream)
    local = ps.finalize(stream=stream)
    if stream is not None:
        torch.cuda.current_stream().wait_stream(stream)
    return gather_keys(local, group)


def sharded_pim(bvh, points: torch.Tensor, rank: int, world: int, direction=(0.0, 0.0, 1.0), filtered=False,
                group=None) -> torch.Tensor:
    """Point-in-mesh over this rank's range of the points, then all ranks' object ids
    concatenated in rank order (every rank returns all n results)."""
    from . import api
    n = points.shape[0]
    lo, hi = split_range(n, world, rank)
    obj, _ = api.point_in_mesh(bvh, points[lo:hi].contiguous(), direction=direction, filtered=filtered)
    return gather_ranges(obj, n, rank, world, group)


def gather_ranges(part: torch.Tensor, n: int, rank: int, world: int, group=None) -> torch.Tensor:
    """Every rank's split_range share of an n-element result, all-gathered (shares padded to
    the largest) and concatenated in rank order."""
    import torch.distributed as dist
    m = split_range(n, world, 0)[1]  # rank 0 has the largest share
    padded = torch.zeros(max(m, 1), dtype=part.dtype, device=part.device)
    padded[:part.numel()] = part
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    sizes = [split_range(n, world, r)[1] - split_range(n, world, r)[0] for r in range(world)]
    return torch.cat([p[:k] for p, k in zip(parts, sizes)])
