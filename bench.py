#!/usr/bin/env python3
"""Benchmark of the RaySpace3D query path on one GB300.

Headline workload (the mesh-overlap join): sets A and B of 10,000 level-2 icospheres
each (320 triangles, 480 unique edges), radius log-uniform in [0.5, 2], Haar rotation,
translation uniform in [0, 1000]^3, seed 1, 128^3 grid statistics per set.  One step is
the whole join as the engine runs it: BVH builds of both sets (concurrently, on two
streams) and grid estimate -> pair-table sizing -> broad phase -> edge rays A->B and
B->A -> sorted unique pair list (raytracer_mesh_overlap order).  `value` is seconds per join with the inputs resident in HBM; `e2e` is the same
join through the C ABI with the inputs in pinned host memory copied in, and the pair
list copied out, inside the timed region.

Secondary (reported in `pim`): point-in-mesh parity of 1,000,000 points uniform in
[-1.5, 1.5]^3 against one level-4 icosphere (+Z rays), in Mpts/s.

`--impl reference` times the reference algorithm on the host cores instead: the
reference's OptiX build cannot run on this machine (no OptiX SDK, and the GPU has no
RT cores), so the arm runs the project's CPU port of the same parity / edge-ray tests
(oracle/) with all host threads: each step is one whole join (both CPU BVH builds and
every edge ray of both directions), timed, with the GPU arm's warm-up and step counts.

Every line carries `parity`: its result compared with the oracle's on the same inputs,
outside the timed region.
"""
from __future__ import annotations

import argparse
import atexit
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "overlap-join sec"
UNIT = "s"
WORKLOAD = ("overlap join: 10k + 10k level-2 icospheres, radius log-uniform [0.5,2], "
            "uniform rotation, translation uniform in 1000^3, seed 1, 128^3 grid")
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--objects", type=int, default=10_000)
    ap.add_argument("--world", type=float, default=1000.0)
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--pim-points", type=int, default=1_000_000)
    ap.add_argument("--no-pim", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--batch-full", action="store_true", help="batched workload at its full size")
    ap.add_argument("--learned-full", action="store_true", help="learned estimator at its full size")
    ap.add_argument("--learned-pairs", type=str, default=None,
                    help="TRAIN,HELD_OUT,MAX_OBJECTS dataset pairs of the learned estimator (overrides the default "
                         "240,60,20000 and --learned-full's 2000,200,200000)")
    ap.add_argument("--only-learned", action="store_true", help="run the learned-estimator section alone")
    ap.add_argument("--intersection-n", type=int, default=10_000, help="objects per set of the intersection join")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--leaf", type=int, default=0, help="BVH leaf size of the joins (0: the engine's default, 2)")
    ap.add_argument("--endpoints", choices=["auto", "host", "device"], default="auto",
                    help="end to end: edge payloads read in place from pinned host memory (host), copied (device), "
                         "or chosen per join from its estimate (auto)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def make_workload(args):
    from rayspace3d_gb300 import synth
    cache = os.path.join(tempfile.gettempdir(), f"rs_bench_{args.objects}_{args.world:g}_{args.grid}.npz")
    A, B = synth.overlap_workload(n_objects=args.objects, level=2, world=args.world, seed=1,
                                  grid_resolution=args.grid)
    return A, B


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"rs_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.f, stderr=subprocess.DEVNULL)
            atexit.register(self.__exit__, None, None, None)  # never outlive the bench
            # Sampling is live once the first line is written (nvidia-smi takes a moment to start).
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                self.f.flush()
                if os.path.getsize(self.path) > 0:
                    break
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if getattr(self, "f", None) is not None and not self.f.closed:
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


def live_check_bytes(src):
    """Bytes of one direction's live-edge check: 8 B per edge (offset, count) and 4 B per
    source id, plus one flag byte per source object."""
    e = src.host.edges
    return 8 * len(e.offsets) + 4 * len(e.sources) + int(src.host.tri2obj.max()) + 1


def build_bytes(g):
    """Algorithmic bytes of one BVH build: read vertices/indices/tri2obj, write the
    leaf-ordered triangles (48 B) and the nodes (64 B per internal node)."""
    return 12 * g.nV + 16 * g.nF + 48 * g.nF + 64 * max(g.nF - 1, 1)


def profiled_traffic(kernel: str, objects: int):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu summary
    profiles/<kernel>.md (line `traffic_bytes_per_launch_<objects> = N`), else None."""
    path = os.path.join(ROOT, "profiles", kernel + ".md")
    try:
        for line in open(path):
            line = line.strip().strip("`")
            if line.startswith(f"traffic_bytes_per_launch_{objects} ="):
                return int(float(line.split("=", 1)[1]))
    except (OSError, ValueError):
        pass
    return None


def run_engine(args, rank, world, local):
    import torch
    from rayspace3d_gb300 import _lib, api, synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.load()
    stream = torch.cuda.Stream(device=dev)
    A, B = make_workload(args)
    pairs_out = {}

    sa, sb = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
        torch.cuda.synchronize()

        def step(ga, gb, after_copies=False, edges_ready=None, edges_hook=None):
            # The two builds run concurrently on their own streams (after the work already
            # queued on `stream`, or, end to end, after their own geometry copies); the join
            # on `stream` is ordered after both builds by the engine.
            if not after_copies:
                sa.wait_stream(stream)
                sb.wait_stream(stream)
            ba = api.Bvh(ga, leaf_size=args.leaf, stream=sa, asynchronous=True)
            bb = api.Bvh(gb, leaf_size=args.leaf, stream=sb, asynchronous=True)
            est, _ = api.estimate_pairs(ga, gb, stream=stream)
            indexes = None
            if edges_hook is not None:  # end to end: the edge payloads are queued now
                edges_ready, indexes = edges_hook(est)
            size = api.hash_size_pow2(est)
            key = ("ps", size)
            ps = pairs_out.get(key)
            if ps is not None and ps.info()[0] != size:
                ps.close()  # grown by an earlier join: every join starts from the estimate's size
                ps = None
            if ps is None:
                ps = api.PairSet(size, pow2=True, stream=stream)
                pairs_out[key] = ps
            # End to end, the broad phase runs while the edge payloads are still in flight
            # and each direction's rays wait for their own payload.
            api.overlap_join(ba, bb, ps, stream=stream, edges_ready=edges_ready, indexes=indexes)
            keys = ps.finalize(order=1, stream=stream)
            ba.close()
            bb.close()
            return keys

        # Clocks are sampled from before the warm-up steps until after the end-to-end steps:
        # the timed region alone (K joins of about a millisecond) is shorter than the sampling
        # period.
        clk = Clocks(local).__enter__()
        for _ in range(args.warmup):
            keys = step(da, db)
        torch.cuda.synchronize()
        n_pairs = int(keys.numel())

        # Device-resident timing (inputs > L2: ~487 MB of geometry + 64 MB of grids per step).
        L.rs_profile_reset()
        L.rs_profile_enable(1)
        launches0 = L.rs_launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            keys = step(da, db)
        ev1.record(stream)
        torch.cuda.synchronize()
        launches = L.rs_launch_count() - launches0
        L.rs_profile_enable(0)
        dev_ms = ev0.elapsed_time(ev1) / args.steps
        prof = {}
        for kid, name in enumerate(["edge_join", "containment", "pim", "bvh_build", "finalize", "estimate",
                                    "build_up"]):
            import ctypes
            ms = ctypes.c_double()
            cnt = ctypes.c_uint64()
            L.rs_profile_read(kid, ctypes.byref(ms), ctypes.byref(cnt))
            if cnt.value:
                prof[name] = {"total_ms": ms.value, "launches": cnt.value, "avg_ms": ms.value / cnt.value}

        # End to end through the C ABI with host buffers.
        # Per set: the triangles (vertices, indices, object ids), the edge payload, the grid.
        host = {}

        def tri_tensors(g):
            return [g.V, g.I, g.T]

        for tag, g in (("A", da), ("B", db)):
            host[tag] = {"tri": [t.cpu().pin_memory() for t in tri_tensors(g)],
                         "edges": [t.cpu().pin_memory() for t in g.edges],
                         "cells": g.cells.cpu().pin_memory()}
        # The edge payloads either stay in pinned host memory, where the join reads in place
        # only the slabs of 256 edges that can hold an edge of an object with a partner (each
        # set's slab index, 3 + nE / 256 int64, is built once per dataset like its grid and
        # copied with the grids), or are copied whole.  In place pays while few objects have
        # partners: about two per estimated pair, each object's x-slab of the payload holds
        # roughly edges * (its x extent / the world's), against all edges copied.  It is
        # chosen per join from the join's own estimate: in place while est < objects / 12
        # (W = 1000: in place; W = 80.7, estimate 1,404 for 10k objects: copied).
        in_place_below = max(1, args.objects // 12)
        for tag, g in (("A", da), ("B", db)):
            idx, ordered = api.edge_index(g)
            host[tag]["index"] = idx.cpu().pin_memory()
            host[tag]["ordered"] = ordered
        dev_edges = {tag: tuple(torch.empty_like(t) for t in g.edges) for tag, g in (("A", da), ("B", db))}
        dev_index = {tag: torch.empty_like(host[tag]["index"], device=dev) for tag in ("A", "B")}
        ga2 = api.DeviceGeometry.__new__(api.DeviceGeometry)
        gb2 = api.DeviceGeometry.__new__(api.DeviceGeometry)
        for dst, src in ((ga2, da), (gb2, db)):
            dst.__dict__.update(src.__dict__)
            dst.V, dst.I, dst.T = [torch.empty_like(t) for t in (src.V, src.I, src.T)]
            dst.cells = torch.empty_like(src.cells)
        chosen = []

        def step_h2d(in_place):
            edges = sum(t.numel() * t.element_size() for hs in host.values() for t in hs["edges"])
            return sum(t.numel() * t.element_size() for hs in host.values()
                       for t in hs["tri"] + [hs["cells"], hs["index"]]) + (0 if in_place else edges)

        sc = torch.cuda.Stream(device=dev)
        ev = {k: torch.cuda.Event() for k in ("A", "B", "cells", "edgesA", "edgesB")}

        def e2e_step():
            # All inputs go over one copy stream, in the order the step needs them: each
            # set's triangles (its build starts when they land), the grids and slab indexes
            # (the estimate and the table sizing run while the rest is in flight), then --
            # when this join's estimate says to copy them -- A's and B's edge payloads.
            sc.wait_stream(stream)
            with torch.cuda.stream(sc):
                for dst, tag in ((ga2, "A"), (gb2, "B")):
                    for d, h in zip(tri_tensors(dst), host[tag]["tri"]):
                        d.copy_(h, non_blocking=True)
                    ev[tag].record(sc)
                for dst, tag in ((ga2, "A"), (gb2, "B")):
                    dst.cells.copy_(host[tag]["cells"], non_blocking=True)
                    dev_index[tag].copy_(host[tag]["index"], non_blocking=True)
                ev["cells"].record(sc)
            sa.wait_event(ev["A"])
            sb.wait_event(ev["B"])
            stream.wait_event(ev["cells"])

            def edges_after_estimate(est):
                in_place = args.endpoints == "host" or (args.endpoints == "auto" and est < in_place_below)
                chosen.append(in_place)
                with torch.cuda.stream(sc):
                    for dst, tag in ((ga2, "A"), (gb2, "B")):
                        hs = host[tag]["edges"]
                        dst.edges = tuple(hs) if in_place else dev_edges[tag]
                        if not in_place:
                            for d, h in zip(dev_edges[tag], hs):
                                d.copy_(h, non_blocking=True)
                        ev["edges" + tag].record(sc)
                return (ev["edgesA"], ev["edgesB"]), ((dev_index["A"], dev_index["B"]) if in_place else None)

            k = step(ga2, gb2, after_copies=True, edges_hook=edges_after_estimate)
            out = k.cpu()
            return out

        for _ in range(max(1, args.warmup // 2)):
            out = e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            out = e2e_step()
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
        d2h = int(out.numel() * out.element_size())
        in_place = chosen[-1]
        h2d = step_h2d(in_place)
        clk.__exit__(None, None, None)

    # Parity spot check of this run's output against the previous device-resident result.
    assert int(out.numel()) == n_pairs
    with torch.cuda.stream(stream):
        rc = recheck(L, lambda: (step(da, db), torch.cuda.synchronize()))

    # Roofline of the join's dominant kernel by the launch list, k_build_tree (the triangles
    # in leaf order and the tree of each BVH build; two launches per join, one per set, on
    # two concurrent streams).  Algorithmic bytes per launch: the set's triangles read once (12 B per
    # vertex, 16 B index triple and object id per triangle), the sorted 8 B keys, the 48 B
    # leaf-ordered triangles written, and 64 B for each tree node over more than
    # leaf_size triangles (at least nF / leaf_size - 1 of them).
    hbm, peak_kind = peaks()
    roof = None
    p = prof.get("build_up")
    if p:
        leaf = 2
        per_launch = sum(12.0 * g.nV + (16.0 + 8.0 + 48.0) * g.nF + 64.0 * (g.nF / leaf - 1) for g in (da, db)) / 2.0
        achieved = per_launch / (p["avg_ms"] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": "k_build_tree", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 5), "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
                "algorithmic_bytes_per_launch": int(per_launch), "avg_launch_ms": round(p["avg_ms"], 4),
                "traffic": profiled_traffic("k_build_tree", args.objects)}
    # The edge rays of one join (the live-edge check of both directions in one launch, then
    # each direction's rays for its live edges, the two directions concurrently; one timed
    # interval per join).  Algorithmic bytes: what the interval has to read with the broad
    # phase's object flags in hand -- each direction's per-edge offset and count (8 B) and
    # 4 B per source id, one flag byte per object -- and 8 B per pair-table insert; the few
    # live edges' endpoints and the nodes their rays visit are left out (mostly L2 hits).
    roof_edges = None
    p = prof.get("edge_join")
    if p:
        per_launch = sum(live_check_bytes(g) for g in (da, db)) + 8.0 * n_pairs
        achieved = per_launch / (p["avg_ms"] * 1e-3) / 1e9
        roof_edges = {"bound": "hbm",
                      "kernel": "k_edge_live + k_edge_rays_warp / k_edge_rays + k_edge_long_warp (both directions)",
                      "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 5),
                      "algorithmic_bytes_per_launch": int(per_launch), "avg_launch_ms": round(p["avg_ms"], 4),
                      "traffic": profiled_traffic("edge_rays_w1000", args.objects)}

    result = {
        "metric": METRIC, "value": round(dev_ms / 1e3, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (exact-sign predicates, FP64 fallback)",
        "data": "synthetic (seeded icospheres; no public dataset is named)",
        "config": {"workload": WORKLOAD, "objects_per_set": args.objects, "world": args.world,
                   "edges_per_set": int(da.nE), "triangles_per_set": int(da.nF), "pairs": n_pairs,
                   "l2": "inputs larger than L2 (geometry ~487 MB + grids 64 MB per step)",
                   "bvh_leaf_size": args.leaf or 2, "parallelism": f"independent joins per rank x{world}"},
        "e2e": {"value": round(e2e_s, 6), "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": d2h,
                "edge_payloads": (("pinned host memory, read in place by the join: only the slabs of objects "
                                   "with partners (slab indexes copied)") if in_place else "copied") +
                                 f" (--endpoints {args.endpoints}; auto: in place while the estimate is below "
                                 f"{in_place_below} pairs)"},
        "gpu_launches": int(launches),
        # The workload's second metric: edge rays of both directions (2 x edges per set) per
        # second of join; the broad phase traces only the live ones.
        "edge_rays_mrays_s": round((da.nE + db.nE) / (dev_ms * 1e-3) / 1e6, 1),
        "recheck": rc,
        "kernels": {k: {kk: round(vv, 5) if isinstance(vv, float) else vv for kk, vv in v.items()}
                    for k, v in prof.items()},
        "roofline": roof,
        "roofline_edge_rays": roof_edges,
        "clocks": dict(clk.summary(), window="warm-up, timed and end-to-end joins"),
        "_keys": out.numpy().view(np.uint64),
    }
    return result, A, B


def recheck(L, fn):
    """Runs fn once with triangle-test counting on; returns the recheck statistics."""
    import ctypes
    L.rs_recheck_reset()
    L.rs_recheck_enable(1)
    try:
        fn()
    finally:
        L.rs_recheck_enable(0)
    ex, tests = ctypes.c_uint64(), ctypes.c_uint64()
    L.rs_recheck_read(ctypes.byref(ex), ctypes.byref(tests))
    return {"exact_edge_signs": ex.value, "triangle_tests": tests.value,
            "rate_per_test": (ex.value / tests.value) if tests.value else 0.0}


def run_pim(args, local, n_points, direction, reps=20, filtered=False, cpu=False):
    """Point-in-mesh on one level-4 icosphere: kernel time (profiler), stream time and
    end-to-end time with the points copied in from pinned host memory.  filtered: the
    filter-refine variant (bounding-box mesh test first, raytracer_filter_refine)."""
    import ctypes

    import torch
    from rayspace3d_gb300 import _lib, api, synth

    L = _lib.load()
    g, pts = synth.pim_workload(n_points, level=4, seed=0)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        dg = api.DeviceGeometry(g)
        bvh = api.Bvh(dg, stream=stream)
        dp = torch.from_numpy(pts).cuda()
        obj = torch.empty(len(pts), dtype=torch.int32, device="cuda")
        inside = torch.empty(len(pts), dtype=torch.uint8, device="cuda")
        for _ in range(3):
            api.point_in_mesh(bvh, dp, direction=direction, filtered=filtered, out_obj=obj, out_inside=inside,
                              stream=stream)
        torch.cuda.synchronize()
        L.rs_profile_reset()
        L.rs_profile_enable(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            api.point_in_mesh(bvh, dp, direction=direction, filtered=filtered, out_obj=obj, out_inside=inside,
                              stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        L.rs_profile_enable(0)
        ms = e0.elapsed_time(e1) / reps
        kms = ctypes.c_double()
        cnt = ctypes.c_uint64()
        L.rs_profile_read(2, ctypes.byref(kms), ctypes.byref(cnt))
        kavg = kms.value / max(cnt.value, 1)
        hp = torch.from_numpy(pts).pin_memory()
        hin = torch.empty(len(pts), dtype=torch.uint8).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            dp.copy_(hp, non_blocking=True)
            api.point_in_mesh(bvh, dp, direction=direction, filtered=filtered, out_obj=obj, out_inside=inside,
                              stream=stream)
            hin.copy_(inside, non_blocking=True)
        torch.cuda.synchronize()
        e2e = (time.perf_counter() - t0) / reps
        rc = recheck(L, lambda: (api.point_in_mesh(bvh, dp, direction=direction, filtered=filtered, out_obj=obj,
                                                   out_inside=inside, stream=stream), torch.cuda.synchronize()))
    hbm, kind = peaks()
    nbytes = 13 * len(pts) + 12 * dg.nV + 16 * dg.nF
    axis = "xyz"[int(np.argmax(np.abs(direction)))]
    extra = {}
    if cpu:
        # Parity of this run's objects against the oracle, and the oracle's own rate on
        # the host cores over the same points (the CPU baseline).
        got = obj.cpu().numpy()
        t_cpu, want = cpu_pim(g, pts, direction, filtered)
        extra["parity"] = parity_of(got, want, f"object id of all {len(pts)} points")
        extra["cpu_baseline"] = {"value": round(len(pts) / t_cpu / 1e6, 2), "unit": "Mpts/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": f"all {len(pts)} points, one pass"}
    return {**extra,
            "workload": f"{len(pts)} points uniform in [-1.5,1.5]^3, level-4 icosphere (5120 triangles), "
                        f"+{axis} rays, seed 0" + (", bounding-box filter then refine" if filtered else ""),
            "mpts_s": round(len(pts) / (ms * 1e-3) / 1e6, 2), "ms": round(ms, 4),
            "kernel_ms": round(kavg, 4), "inside_frac": round(float((obj >= 0).float().mean().item()), 5),
            "e2e_mpts_s": round(len(pts) / e2e / 1e6, 2),
            "e2e_bytes_per_call": {"h2d": 12 * len(pts), "d2h": len(pts)},
            "recheck": rc,
            "roofline": {"bound": "hbm", "achieved": round(nbytes / (kavg * 1e-3) / 1e9, 2), "peak": hbm,
                         "unit": "GB/s", "frac": round(nbytes / (kavg * 1e-3) / 1e9 / hbm, 5),
                         "algorithmic_bytes_per_launch": nbytes, "peak_source": kind + " hbm_gbs"}}


def run_join_variant(args, world_size, steps=5, filtered=False, cpu=False):
    """The overlap join at another world size (device-resident), pairs and recheck rate.
    filtered: the same join through rs_overlap_join_filtered (object-box filter, BVHs over
    the overlapping objects' triangles only, built inside the call)."""
    import torch
    from rayspace3d_gb300 import _lib, api, synth

    L = _lib.load()
    A, B = synth.overlap_workload(n_objects=args.objects, level=2, world=world_size, seed=1,
                                  grid_resolution=args.grid)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
        cache = {}

        sa, sb = torch.cuda.Stream(), torch.cuda.Stream()

        def step():
            est, _ = api.estimate_pairs(da, db, stream=stream)
            size = api.hash_size_pow2(est)
            ps = cache.get(size)
            if ps is not None and ps.info()[0] != size:
                ps.close()  # grown by an earlier join: every join starts from the estimate's size
                ps = None
            if ps is None:
                ps = cache[size] = api.PairSet(size, pow2=True, stream=stream)
            if filtered:
                api.overlap_join_filtered(da, db, ps, stream=stream)
                return ps.finalize(order=1, stream=stream), est
            sa.wait_stream(stream)
            sb.wait_stream(stream)
            ba, bb = api.Bvh(da, stream=sa, asynchronous=True), api.Bvh(db, stream=sb, asynchronous=True)
            api.overlap_join(ba, bb, ps, stream=stream)
            keys = ps.finalize(order=1, stream=stream)
            ba.close()
            bb.close()
            return keys, est

        for _ in range(3):
            keys, est = step()
        torch.cuda.synchronize()
        L.rs_profile_reset()
        L.rs_profile_enable(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            keys, est = step()
        e1.record(stream)
        torch.cuda.synchronize()
        L.rs_profile_enable(0)
        ms = e0.elapsed_time(e1) / steps
        prof = {}
        for kid, name in ((0, "edge_rays"), (6, "build_up")):
            import ctypes
            kms, cnt = ctypes.c_double(), ctypes.c_uint64()
            L.rs_profile_read(kid, ctypes.byref(kms), ctypes.byref(cnt))
            if cnt.value:
                prof[name] = {"avg_ms": round(kms.value / cnt.value, 5), "launches": cnt.value}
        rc = recheck(L, lambda: (step(), torch.cuda.synchronize()))
    n_pairs = int(keys.numel())
    out = {"workload": f"overlap join: {args.objects} + {args.objects} level-2 icospheres, world {world_size:g}^3, "
                       f"seed 1, {args.grid}^3 grid" + (", object-filtered BVHs" if filtered else ""),
           "seconds": round(ms / 1e3, 6), "pairs": n_pairs, "estimated_pairs": int(est),
           "selectivity": n_pairs / float(args.objects) ** 2,
           "edge_rays_per_join": int(da.nE + db.nE), "recheck": rc, "kernels": prof}
    p = prof.get("edge_rays")
    if p and not filtered:
        # The edge rays of one join (broad-phase live check, binning, fast and deferred ray
        # kernels of both directions; one timed interval per join), with the algorithmic bytes
        # of the headline's edge interval: the live check's per-edge read and 8 B per pair.
        # At this selectivity the rays themselves dominate: a divergent, latency-bound
        # traversal whose node reads mostly hit L2, so the fraction is low by construction.
        hbm, kind = peaks()
        nbytes = sum(live_check_bytes(g) for g in (da, db)) + 8.0 * n_pairs
        ach = nbytes / (p["avg_ms"] * 1e-3) / 1e9
        out["roofline"] = {"bound": "hbm", "kernel": "edge rays of both directions (k_edge_live .. k_edge_long_warp)",
                           "achieved": round(ach, 2), "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 5),
                           "algorithmic_bytes_per_launch": int(nbytes), "avg_launch_ms": p["avg_ms"],
                           "peak_source": kind + " hbm_gbs", "traffic": None}
    if cpu:
        t_cpu, want = cpu_join(A, B)
        out["parity"] = parity_of(keys.cpu().numpy().view(np.uint64), key_order1(want),
                                  "sorted pair list (raytracer_mesh_overlap order)")
        if not filtered:
            out["cpu_baseline"] = {"value": round(t_cpu, 4), "unit": "s", "cores": os.cpu_count(), "kind": "port",
                                   "sample": f"one whole join: {len(A.edges.starts)} + {len(B.edges.starts)} edge rays "
                                             f"and both CPU BVH builds"}
    return out


def run_batch(args, full: bool):
    """The batched, degeneracy-heavy configuration in one persistent launch (rs_batch_*):
    256 point-in-mesh queries over meshes of 80..81,920 triangles (icosphere levels 1-6,
    and face-sharing cube blocks), point counts log-uniform in [1e4, 4e6] (full) or
    [1e4, 1e6] (default), 20 % snapped onto vertices, edges and faces, +x/+y/+z and
    oblique rays; plus both edge directions of 64 (full) or 16 (default) overlap joins of
    level-2 icospheres, objects per side log-uniform in [1e3, 5e4] (full) or [1e3, 2e4],
    world scaled to the 10k-in-1000^3 density, one in eight a pair of face-sharing cube
    blocks offset by half a cube.  Everything is generated on the device (gen.py).  The
    autotuner picks leaf size, chunk and stack depth first; then the batch is replayed
    as a CUDA graph and timed.  A sample of queries is checked against the
    single-query entry points."""
    import ctypes

    import torch
    from rayspace3d_gb300 import _lib, api, gen, synth

    L = _lib.load()
    rng = np.random.default_rng(4)
    n_pim, n_join = 256, (64 if full else 16)
    pmax, omax = (4e6, 5e4) if full else (1e6, 2e4)
    keep = []
    meshes = []
    queries = []  # (mesh index, points, direction)
    for q in range(n_pim):
        if q % 10 == 9:
            nx, ny, nz = (int(v) for v in rng.integers(1, 9, size=3))
            g = synth.cube_grid(nx, ny, nz, edges=False)
            dg = api.DeviceGeometry(g)
        else:
            level = int(rng.integers(1, 7))
            dg = gen.instanced_set(1, level, 1.0, 1.0, 0.0, seed=1000 + q)
        meshes.append(dg)
        n = int(np.exp(rng.uniform(np.log(1e4), np.log(pmax))))
        pts = gen.mesh_points(dg, n, seed=2000 + q, frac_snapped=0.2)
        k = q % 4
        d = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), None][k]
        if d is None:
            v = rng.standard_normal(3)
            v /= np.linalg.norm(v)
            d = tuple(float(x) for x in v)
        queries.append((q, pts, d))
    joins = []
    for j in range(n_join):
        if j % 8 == 7:
            A = api.DeviceGeometry(synth.cube_grid(20, 20, 5))
            gb = synth.cube_grid(20, 20, 5)
            gb = synth.make_geometry(gb.vertices + np.float32(0.5), gb.indices, gb.tri2obj)
            B = api.DeviceGeometry(gb)
        else:
            n = int(np.exp(rng.uniform(np.log(1e3), np.log(omax))))
            w = 1000.0 * (n / 1e4) ** (1.0 / 3.0)
            A = gen.instanced_set(n, 2, 0.5, 2.0, w, seed=3000 + 2 * j)
            B = gen.instanced_set(n, 2, 0.5, 2.0, w, seed=3001 + 2 * j)
        joins.append((A, B))
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        bvhs = [api.Bvh(dg, stream=stream) for dg in meshes]
        jb = [(api.Bvh(A, stream=stream), api.Bvh(B, stream=stream)) for A, B in joins]
        sets = [api.PairSet(1 << 20, stream=stream) for _ in joins]
        outs = []
        h = ctypes.c_void_p()
        L.rs_batch_create(ctypes.byref(h))
        for (q, pts, d) in queries:
            obj = torch.empty(len(pts), dtype=torch.int32, device="cuda")
            ins = torch.empty(len(pts), dtype=torch.uint8, device="cuda")
            L.rs_batch_add_pim(h, bvhs[q].handle, pts.data_ptr(), len(pts), *d, obj.data_ptr(), ins.data_ptr(), None)
            outs.append((obj, ins))
        for (A, B), (ba, bb), ps in zip(joins, jb, sets):
            L.rs_batch_add_edges(h, bb.handle, *A.edge_ptrs(), A.nE, 0, ps.handle, None)
            L.rs_batch_add_edges(h, ba.handle, *B.edge_ptrs(), B.nE, 1, ps.handle, None)
        sp = ctypes.c_void_p(stream.cuda_stream)
        leaf, ch, sd, tms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        t0 = time.perf_counter()
        rc_tune = L.rs_batch_autotune(h, ctypes.byref(leaf), ctypes.byref(ch), ctypes.byref(sd), ctypes.byref(tms),
                                      sp)
        tune_s = time.perf_counter() - t0
        nq = n_pim + 2 * n_join
        st = (ctypes.c_int * nq)()
        for ps in sets:
            ps.clear(stream=stream)
        rc = L.rs_batch_submit(h, sp)  # captures the graph
        rc = rc or L.rs_batch_wait(h, st)
        reps = 5
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            L.rs_batch_submit(h, sp)
        e1.record(stream)
        rc = rc or L.rs_batch_wait(h, st)
        ms = e0.elapsed_time(e1) / reps
        rc_stats = recheck(L, lambda: (L.rs_batch_submit(h, sp), L.rs_batch_wait(h, st)))
        # Spot checks against the single-query entry points.
        checks = 0
        for i in list(range(0, n_pim, 37)):
            q, pts, d = queries[i]
            o, _ = api.point_in_mesh(bvhs[q], pts, direction=d, stream=stream)
            torch.cuda.synchronize()
            assert torch.equal(o, outs[i][0]), f"batch point-in-mesh query {i} differs"
            checks += 1
        for j in list(range(0, n_join, 5)) + [7]:
            if j >= n_join:
                continue
            ref = api.PairSet(1 << 20, stream=stream)
            api.overlap_join(jb[j][0], jb[j][1], ref, stream=stream)
            a = ref.finalize(stream=stream).cpu().numpy()
            b = sets[j].finalize(stream=stream).cpu().numpy()
            assert np.array_equal(np.sort(a), np.sort(b)), f"batch join {j} differs"
            checks += 1
        L.rs_batch_destroy(h)
    n_pts = sum(len(p) for _, p, _ in queries)
    n_edges = sum(A.nE + B.nE for A, B in joins)
    n_tris_join = sum(A.nF + B.nF for A, B in joins)
    return {"workload": ("full" if full else "default") + f": {n_pim} point-in-mesh queries ({n_pts} points, "
                        f"20 % snapped) + {n_join} overlap joins ({n_edges} edge rays, {n_tris_join} triangles), "
                        "one persistent launch replayed as a CUDA graph",
            "status": int(rc), "ms": round(ms, 3), "mrays_s": round((n_pts + n_edges) / (ms * 1e-3) / 1e6, 1),
            "points": int(n_pts), "edge_rays": int(n_edges),
            "autotune": {"status": int(rc_tune), "leaf_size": leaf.value, "chunk": ch.value,
                         "stack_depth": sd.value, "best_ms": round(tms.value, 3), "seconds": round(tune_s, 2)},
            "recheck": rc_stats, "spot_checks_passed": checks}


def run_intersection(args, n: int):
    """Full intersection join at uneven sizes: n objects per set (10k by default, the
    configuration's 100k with --intersection-n 100000) of icospheres with levels 1..5
    (triangle counts log-uniform), radii log-uniform in [0.2, 20], uniform in a 2000^3
    world (scaled to keep the density at smaller n), seed 2, 5 % of B planted strictly
    inside A objects.  One step = both BVH builds (concurrent) + overlap both ways +
    containment both ways + sorted pair list.  The device memory the step needs (both
    BVHs at 112 B per triangle and the builds' scratch) is checked against the free memory
    after generation; a size that does not fit is reported as skipped."""
    import torch
    from rayspace3d_gb300 import api, gen

    world = 2000.0 * (n / 100_000) ** (1.0 / 3.0)
    t0 = time.perf_counter()
    A, B, planted = gen.intersection_sets(n, seed=2, world=world)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    torch.cuda.empty_cache()  # generation temporaries back to the driver for the builds
    free0, total = torch.cuda.mem_get_info()
    # BVH 112 B/triangle resident per set; per build in flight: keys and their copy 16 B,
    # sort status 0.7 B, open subtrees <= 18 B, exchange 4 B per triangle.
    need = 112 * (A.nF + B.nF) + 39 * (A.nF + B.nF) + 8 * (A.nE + B.nE)
    if need > 0.97 * free0:
        return {"workload": f"full intersection: {n} + {n} objects", "skipped":
                f"needs about {need / 1e9:.0f} GB of device memory, {free0 / 1e9:.0f} GB free after generation"}
    stream = torch.cuda.Stream()
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ps = api.PairSet(1 << 20, stream=stream)

        def step():
            sa.wait_stream(stream)
            sb.wait_stream(stream)
            ba, bb = api.Bvh(A, stream=sa, asynchronous=True), api.Bvh(B, stream=sb, asynchronous=True)
            ps.clear(stream=stream)
            api.overlap_join(ba, bb, ps, with_containment=True, stream=stream)
            keys = ps.finalize(stream=stream)
            ba.close()
            bb.close()
            return keys

        keys = step()
        torch.cuda.synchronize()
        steps = 3
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            keys = step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
    k = keys.cpu().numpy().astype(np.uint64)
    ks = set(int(x) for x in k)
    found = sum(((a << 32) | b) in ks for a, b in planted)
    return {"workload": f"full intersection: {n} + {n} icospheres of levels 1..5, radii 0.2..20, world {world:.0f}^3, "
                        f"seed 2, {len(planted)} B objects planted inside A",
            "seconds": round(ms / 1e3, 5), "pairs": int(len(k)), "planted_found": int(found),
            "planted": len(planted), "triangles_per_set": [int(A.nF), int(B.nF)],
            "edge_rays": int(A.nE + B.nE), "generation_s": round(gen_s, 1),
            "device_gb": {"inputs": round((total - free0) / 1e9, 1),
                          "peak_in_use": round((total - torch.cuda.mem_get_info()[0]) / 1e9, 1),
                          "total": round(total / 1e9, 1)}}


def run_learned(args, full: bool):
    """Learned selectivity estimator: dataset pairs (mixture-placed icospheres and boxes,
    radii log-uniform in [0.1, 50], 1000^3 world; 1k..200k objects per side in the full
    run, 1k..20k by default), labelled by the engine's exact joins; train on all but the
    held-out pairs; errors of the network and of the grid estimator on the held-out ones;
    tensor-core throughput of the forward pass (bound: BF16 tensor peak)."""
    import ctypes

    import torch
    from rayspace3d_gb300 import _lib, learned

    n_train, n_test = (2000, 200) if full else (240, 60)
    n_hi = 200_000 if full else 20_000
    if getattr(args, "learned_pairs", None):
        n_train, n_test, n_hi = (int(x) for x in args.learned_pairs.split(","))
    t0 = time.perf_counter()
    samples = [learned.make_sample(10_000 + i, 1000, n_hi) for i in range(n_train + n_test)]
    gen_s = time.perf_counter() - t0
    train, test = samples[:n_train], samples[n_train:]
    t0 = time.perf_counter()
    # The network corrects the grid estimate; weight decay, early stopping on the last 15 %
    # of the training pairs, symmetry augmentation (learned.train).
    m, losses = learned.train(train, epochs=40 if full else 80, batch=64, lr=1e-3, seed=0, prior=True,
                              weight_decay=1e-2, val_frac=0.15)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    ev_test = learned.evaluate(m, test)
    ev_train = learned.evaluate(m, train)
    # Forward-pass throughput (2 * (32768*512 + 512*512 + 512) flop per row) and the two
    # GEMMs alone (device time of the GEMM launches and their split-K sums, CUDA events on the
    # launching stream).  At 256 rows the first GEMM streams W1 (32 MB) for 8.6 GFLOP, below
    # the machine balance: bound by HBM.  At 4096 rows (a whole evaluation set per pass) it
    # is bound by the tensor cores.
    L0 = _lib.load()

    def forward_rates(B, reps=20):
        X = torch.rand((B, learned.N_FEAT), device="cuda")
        for _ in range(3):
            m.forward(X)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            m.forward(X)
        e1.record()
        torch.cuda.synchronize()
        fms = e0.elapsed_time(e1) / reps
        L0.rs_profile_reset()
        L0.rs_profile_enable(1)
        for _ in range(reps):
            m.forward(X)
        torch.cuda.synchronize()
        gms, gcnt = ctypes.c_double(), ctypes.c_uint64()
        L0.rs_profile_read(7, ctypes.byref(gms), ctypes.byref(gcnt))
        L0.rs_profile_enable(0)
        g = gms.value / reps if gcnt.value else None
        del X
        return fms, g

    B = 256
    ms, gemm_ms = forward_rates(B)
    tflops = 2.0 * B * (32768 * 512 + 512 * 512 + 512) / (ms * 1e-3) / 1e12
    gemm_tflops = (2.0 * B * (32768 * 512 + 512 * 512)) / (gemm_ms * 1e-3) / 1e12 if gemm_ms else None
    # Bytes the 256-row GEMMs must move: X (BF16) and W1 once, W2, the split-K workspace is
    # not counted.
    gemm_bytes = 2.0 * (B * 32768 + 512 * 32768 + 512 * 512 + B * 512)
    BL = 4096
    ms_l, gemm_ms_l = forward_rates(BL, reps=10)
    gemm_tflops_l = (2.0 * BL * (32768 * 512 + 512 * 512)) / (gemm_ms_l * 1e-3) / 1e12 if gemm_ms_l else None
    peak = None
    try:
        with open(MEASURED_PEAKS) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except Exception:
        peak = 1900.0
    # Estimator latency: grid estimator vs network, one pair.
    s0 = test[0]
    L = _lib.load()
    rng = np.random.default_rng(10_000 + n_train)
    A, na = learned.dataset_side(4 * (10_000 + n_train), 1000, n_hi, rng)
    Bs, nb = learned.dataset_side(4 * (10_000 + n_train) + 3, 1000, n_hi, rng)
    ca, cb = learned.grid_cells(A, na), learned.grid_cells(Bs, nb)
    est, lg = ctypes.c_int64(), ctypes.c_double()
    from rayspace3d_gb300 import api
    for _ in range(3):
        L.rs_estimate_mlp(m.h, ca.data_ptr(), cb.data_ptr(), learned.RES, ctypes.byref(est), ctypes.byref(lg), None)
        api.estimate_grid(ca, cb, learned.RES ** 3, learned._cell_volume())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(20):
        L.rs_estimate_mlp(m.h, ca.data_ptr(), cb.data_ptr(), learned.RES, ctypes.byref(est), ctypes.byref(lg), None)
    mlp_ms = (time.perf_counter() - t0) / 20 * 1e3
    t0 = time.perf_counter()
    for _ in range(20):
        api.estimate_grid(ca, cb, learned.RES ** 3, learned._cell_volume())
    grid_ms = (time.perf_counter() - t0) / 20 * 1e3
    # End-to-end join time on held-out pairs with the pair table sized from each estimate,
    # and from the true count (the floor): an under-estimate costs table growth and a rerun,
    # an over-estimate a larger table to clear and scan.
    mlp_est = learned.predict(m, test)
    n_join = min(len(test), 30)
    jt = {"mlp": 0.0, "grid": 0.0, "true_count": 0.0}
    for i in range(n_join):
        seed = 10_000 + n_train + i
        jt["mlp"] += learned.join_seconds(seed, mlp_est[i], 1000, n_hi)
        jt["grid"] += learned.join_seconds(seed, test[i].grid_estimate, 1000, n_hi)
        jt["true_count"] += learned.join_seconds(seed, test[i].pairs, 1000, n_hi)
    m.close()
    return {"workload": f"{n_train} training + {n_test} held-out dataset pairs, 1000..{n_hi} objects per side, "
                        "128^3 grids pooled to 16^3x4 per side, MLP 32768-512-512-1 (BF16 weights, FP32 accumulate) "
                        "correcting the grid estimate",
            "join_seconds_held_out": {"pairs": n_join, **{k: round(v, 5) for k, v in jt.items()}},
            "generation_s": round(gen_s, 1), "train_s": round(train_s, 2), "final_train_loss": round(losses[-1], 4),
            "held_out": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in ev_test.items()},
            "train_set": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in ev_train.items()},
            "estimator_ms": {"mlp": round(mlp_ms, 3), "grid": round(grid_ms, 3)},
            "roofline": {"bound": "tensor", "kernel": "k_umma_gemm (tcgen05.mma bf16 into tensor memory, TMA "
                                                          "128B-swizzled operands, split K) + its split sums, the "
                                                          f"forward pass's two GEMMs at B={BL}",
                         "achieved": round(gemm_tflops_l, 2) if gemm_tflops_l else None, "peak": peak,
                         "unit": "TFLOP/s", "frac": round(gemm_tflops_l / peak, 5) if gemm_tflops_l else None,
                         "gemm_ms": round(gemm_ms_l, 4) if gemm_ms_l else None,
                         "forward_pass": {"rows": BL, "ms": round(ms_l, 4)}},
            "roofline_b256": {"bound": "hbm", "kernel": "the same two GEMMs at B=256 (streaming W1)",
                              "achieved": round(gemm_bytes / (gemm_ms * 1e-3) / 1e9, 2) if gemm_ms else None,
                              "peak": peaks()[0], "unit": "GB/s",
                              "frac": round(gemm_bytes / (gemm_ms * 1e-3) / 1e9 / peaks()[0], 5) if gemm_ms else None,
                              "gemm_ms": round(gemm_ms, 4) if gemm_ms else None,
                              "tflops": round(gemm_tflops, 2) if gemm_tflops else None,
                              "forward_pass": {"rows": B, "ms": round(ms, 4), "tflops": round(tflops, 2)}}}


def run_prep(A, cpu: bool = True):
    """GPU preprocessing of one overlap-join set (3.2 M triangles of the headline
    workload): the unique-edge payload (rs_extract_edges) and 128^3 grid statistics over
    the 1000^3 world (rs_grid_stats), both bit-identical to the reference's CPU code, timed
    wall-clock per call with the triangles resident on the device; beside them the same
    two steps by the single-threaded C++ restatement of the reference (std::map /
    std::unordered_map, as the reference runs them), on the full set."""
    import ctypes

    import torch
    from rayspace3d_gb300 import _lib, api

    dg = api.DeviceGeometry(A)
    L = _lib.load()
    cells = torch.empty(128 ** 3 * 16, dtype=torch.uint8, device="cuda")
    b = (ctypes.c_float * 6)()

    def grid():
        api._check(L.rs_grid_stats(dg.V.data_ptr(), dg.nV, dg.I.data_ptr(), dg.nF, dg.T.data_ptr(),
                                   int(dg.T.max().item()) + 1, 128, 1000.0, cells.data_ptr(), b, None),
                   "rs_grid_stats")

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)

    t_edges = timed(lambda: api.extract_edges(dg.V, dg.I, dg.T))
    t_grid = timed(grid)
    e = api.extract_edges(dg.V, dg.I, dg.T)
    out = {"workload": "preprocessing of one overlap-join set: 10k level-2 icospheres (3.2 M triangles), "
                       "unique edges + 128^3 grid over 1000^3",
           "triangles": int(dg.nF), "edges": int(e[0].shape[0]), "sources": int(e[4].shape[0]),
           "gpu_seconds": {"extract_edges": round(t_edges, 5), "grid_stats": round(t_grid, 5)},
           "gpu_mtris_per_s": round(dg.nF / (t_edges + t_grid) / 1e6, 1)}
    if cpu:
        from oracle import bind
        t0 = time.perf_counter()
        bind.extract_edges(A.vertices, A.indices, A.tri2obj)
        c_edges = time.perf_counter() - t0
        t0 = time.perf_counter()
        bind.grid_stats(A.vertices, A.indices, A.tri2obj, 128, 1000.0)
        c_grid = time.perf_counter() - t0
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": "the full set",
                               "seconds": {"extract_edges": round(c_edges, 3), "grid_stats": round(c_grid, 3)}}
        out["speedup_vs_cpu"] = round((c_edges + c_grid) / (t_edges + t_grid), 1)
    return out


def combine_ranks(result: dict, world: int, device) -> dict:
    """N ranks, each running its own joins (independent units, no data-path collective):
    the step time is the slowest rank's, and whole-job seconds per join is that time
    divided by the N joins completed in it.  The end-to-end value combines the same way."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([result["ms_per_step"], result["e2e"]["value"]], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    slow_ms, slow_e2e = float(t[0].item()), float(t[1].item())
    result["ms_per_step"] = round(slow_ms, 4)
    result["value"] = round(slow_ms / 1e3 / world, 6)
    result["e2e"]["value"] = round(slow_e2e / world, 6)
    return result


def cpu_join(A, B, threads=None):
    """One whole oracle overlap join on the host cores, timed: the CPU BVH of each set and
    every edge ray of both directions (the reference's hit rule).  Returns (seconds, keys)."""
    from oracle import bind
    threads = threads or os.cpu_count()
    t0 = time.perf_counter()
    keys = bind.overlap_join(A, B, threads=threads)
    return time.perf_counter() - t0, keys


def cpu_pim(g, pts, direction, filtered=False, threads=None):
    """The oracle's point-in-mesh over the points on the host cores, timed (seconds, objects)."""
    from oracle import bind
    threads = threads or os.cpu_count()
    t0 = time.perf_counter()
    out = bind.pim(g.vertices, g.indices, g.tri2obj, pts, direction=direction, filtered=filtered, threads=threads)
    return time.perf_counter() - t0, out


def key_order1(keys):
    """Sorted u64 keys (id1 << 32 | id2) reordered by (id2, id1), raytracer_mesh_overlap's order."""
    keys = np.asarray(keys, dtype=np.uint64)
    return keys[np.lexsort((keys >> np.uint64(32), keys & np.uint64(0xffffffff)))]


def parity_of(got, want, what):
    got = np.asarray(got)
    want = np.asarray(want)
    if got.shape != want.shape:
        mism = int(abs(len(got) - len(want)) + np.count_nonzero(got[:min(len(got), len(want))] !=
                                                                want[:min(len(got), len(want))]))
    else:
        mism = int(np.count_nonzero(got != want))
    return {"against": "oracle", "checked": what, "mismatches": mism}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        # The CPU arm has no collective: rank 0 alone runs and prints, the other ranks exit.
        if rank != 0:
            return
        A, B = make_workload(args)
        threads = os.cpu_count()
        for _ in range(args.warmup):
            cpu_join(A, B, threads)
        vals = [cpu_join(A, B, threads)[0] for _ in range(args.steps)]
        v = statistics.median(vals)
        sample = (f"whole joins: {len(A.edges.starts)} + {len(B.edges.starts)} edge rays and both CPU BVH builds "
                  f"per step, median of {args.steps} after {args.warmup} warm-up")
        line = {"impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v * 1e3, 3),
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded icospheres)",
                "config": {"workload": WORKLOAD, "objects_per_set": args.objects, "world": args.world},
                "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "reference OptiX build unavailable on this box (no OptiX SDK; GB300 has no RT cores); "
                        "CPU port of the same exact tests on all host threads"}
        print(json.dumps(line))
        return
    if args.only_learned:
        # The learned-estimator section alone (a profiling and sizing aid; no headline line).
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({"learned": run_learned(args, args.learned_full)}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl")
    result, A, B = run_engine(args, rank, world, local)
    cpu = rank == 0 and not args.no_cpu_baseline
    if not args.no_pim:
        result["pim"] = run_pim(args, local, args.pim_points, (1.0, 0.0, 0.0), cpu=cpu)
        result["pim_z"] = run_pim(args, local, args.pim_points, (0.0, 0.0, 1.0), cpu=cpu)
        result["pim_filtered"] = run_pim(args, local, args.pim_points, (0.0, 0.0, 1.0), filtered=True, cpu=cpu)
        if not args.no_variants:
            result["pim_100m"] = run_pim(args, local, 100_000_000, (1.0, 0.0, 0.0), reps=5, cpu=cpu)
    if not args.no_variants:
        result["join_w80"] = run_join_variant(args, 80.7, cpu=cpu)
        result["join_filtered"] = run_join_variant(args, args.world, filtered=True, cpu=cpu)
        result["join_w80_filtered"] = run_join_variant(args, 80.7, filtered=True, cpu=cpu)
        result["batch"] = run_batch(args, args.batch_full)
        result["learned"] = run_learned(args, args.learned_full)
        result["intersection"] = run_intersection(args, args.intersection_n)
        result["prep"] = run_prep(A, cpu=(rank == 0 and not args.no_cpu_baseline))
    if rank == 0:
        # Parity of the headline join, and its CPU baseline: the oracle's whole join, timed.
        v, want = cpu_join(A, B)
        result["parity"] = parity_of(result.pop("_keys"), key_order1(want),
                                     "sorted pair list of the end-to-end join (raytracer_mesh_overlap order)")
        if not args.no_cpu_baseline:
            result["cpu_baseline"] = {"value": round(v, 4), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                      "sample": f"one whole join: {len(A.edges.starts)} + {len(B.edges.starts)} edge "
                                                f"rays and both CPU BVH builds (not extrapolated)"}
    else:
        result.pop("_keys", None)
    if world > 1:
        combine_ranks(result, world, "cuda")
    if rank == 0:
        print(json.dumps(result))


if __name__ == "__main__":
    main()
