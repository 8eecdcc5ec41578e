"""Python host API over librs.so, shaped like the reference's host layer.

Reference counterparts:
  DeviceGeometry.upload      GeometryUploader::upload + PrecomputedEdgeData::uploadFromGeometry
                             (query/src/geometry/GeometryUploader.cpp:12-34, PrecomputedEdgeData.cpp:5-35)
  Bvh                        OptixAccelerationStructure (query/src/optix/OptixAccelerationStructure.cpp:22-68)
  point_in_mesh              RayLauncher::launch + ResultProcessor (query/src/raytracing/RayLauncher.cpp:44-58)
  filter_refine              FilterRefinePipeline::execute (query/src/raytracing/FilterRefine.cpp:81-122)
  PairSet / overlap_join     executeHashQuery of the estimated mains
                             (query/src/applications/raytracer_overlap_estimated_main.cpp:39-112,
                              raytracer_intersection_estimated_main.cpp:77-176)
  estimate_pairs             estimatePairs (raytracer_overlap_estimated_main.cpp:252-325)
PyTorch supplies device memory and streams only; all compute is in librs.so.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np
import torch

from . import _lib
from .formats import Geometry, Grid

_check = _lib.check


RS_FINALIZE_NO_WAIT = 0x100  # rs_pairset_finalize: return once the small-table path is queued


def _stream(stream: Optional[torch.cuda.Stream] = None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("device tensor expected")
    if not t.is_contiguous():
        raise ValueError("contiguous tensor expected")
    return t.data_ptr()


def _kernel_ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    """A device tensor's or a pinned host tensor's address (kernels read pinned memory in
    place, rs_kernel_pointer)."""
    if t is None:
        return None
    if not (t.is_cuda or t.is_pinned()):
        raise ValueError("device or pinned host tensor expected")
    if not t.is_contiguous():
        raise ValueError("contiguous tensor expected")
    return t.data_ptr()


class DeviceGeometry:
    """One .pre geometry set resident on the GPU (vertices, indices, tri2obj, edges, grid)."""

    def __init__(self, g: Geometry, device: str = "cuda"):
        self.host = g
        dev = torch.device(device)
        self.V = torch.from_numpy(np.ascontiguousarray(g.vertices, np.float32)).to(dev)
        self.I = torch.from_numpy(np.ascontiguousarray(g.indices, np.uint32).view(np.int32)).to(dev)
        self.T = torch.from_numpy(np.ascontiguousarray(g.tri2obj, np.int32)).to(dev)
        self.nV = int(len(g.vertices))
        self.nF = int(len(g.indices))
        self.edges = None
        if g.edges is not None and len(g.edges.starts):
            e = g.edges
            self.edges = (torch.from_numpy(np.ascontiguousarray(e.starts, np.float32)).to(dev),
                          torch.from_numpy(np.ascontiguousarray(e.ends, np.float32)).to(dev),
                          torch.from_numpy(np.ascontiguousarray(e.offsets, np.int32)).to(dev),
                          torch.from_numpy(np.ascontiguousarray(e.counts, np.int32)).to(dev),
                          torch.from_numpy(np.ascontiguousarray(e.sources, np.int32)).to(dev))
            self.nE = int(len(e.starts))
        else:
            self.nE = 0
        self.cells = None
        if g.grid is not None:
            raw = np.ascontiguousarray(g.grid.cells).view(np.uint8)
            self.cells = torch.from_numpy(raw.copy()).to(dev)

    @classmethod
    def from_tensors(cls, V: torch.Tensor, I: torch.Tensor, T: torch.Tensor, edges=None,
                     cells: Optional[torch.Tensor] = None) -> "DeviceGeometry":
        """Wraps device tensors (float32 V[n,3], int32/uint32-bits I[m,3], int32 T[m], optional
        edge tuple (starts, ends, offsets, counts, sources) and raw grid cells) without copies."""
        self = cls.__new__(cls)
        self.host = None
        self.V, self.I, self.T = V.contiguous(), I.contiguous(), T.contiguous()
        self.nV, self.nF = int(V.shape[0]), int(I.shape[0])
        self.edges = tuple(t.contiguous() for t in edges) if edges is not None else None
        self.nE = int(self.edges[0].shape[0]) if self.edges is not None else 0
        self.cells = cells
        return self

    def edge_ptrs(self):
        if self.edges is None:
            raise ValueError("geometry has no precomputed edge payload")
        return [t.data_ptr() for t in self.edges]

    def host_tri2obj(self) -> np.ndarray:
        """The object id of every triangle on the host."""
        if getattr(self, "host", None) is not None:
            return np.asarray(self.host.tri2obj)
        return self.T.cpu().numpy()


class Bvh:
    """Engine-owned BVH over a DeviceGeometry (which must stay alive)."""

    def __init__(self, geom: DeviceGeometry, leaf_size: int = 0, stream=None, asynchronous: bool = False):
        """asynchronous=True queues the build on `stream` and returns at once (rs_bvh_build_async);
        queries are ordered after it, wait() reports its status."""
        self.geom = geom
        h = ctypes.c_void_p()
        L = _lib.load()
        fn = L.rs_bvh_build_async if asynchronous else L.rs_bvh_build
        _check(fn(_ptr(geom.V), geom.nV, _ptr(geom.I), geom.nF, _ptr(geom.T), leaf_size, ctypes.byref(h),
                  _stream(stream)), "rs_bvh_build")
        self.handle = h

    def wait(self):
        _check(_lib.load().rs_bvh_wait(self.handle), "rs_bvh_wait")

    def info(self):
        nt, nn, nb = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        mn = (ctypes.c_float * 3)()
        mx = (ctypes.c_float * 3)()
        _check(_lib.load().rs_bvh_info(self.handle, ctypes.byref(nt), ctypes.byref(nn), ctypes.byref(nb), mn, mx),
               "rs_bvh_info")
        return {"triangles": nt.value, "nodes": nn.value, "bytes": nb.value, "min": list(mn), "max": list(mx)}

    def close(self):
        if self.handle:
            _lib.load().rs_bvh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def point_in_mesh(bvh: Bvh, points: torch.Tensor, direction=(0.0, 0.0, 1.0), filtered: bool = False,
                  out_obj: Optional[torch.Tensor] = None, out_inside: Optional[torch.Tensor] = None,
                  stream=None) -> Tuple[torch.Tensor, torch.Tensor]:
    """Object of the first counted hit (or -1) and the inside bit for each point (float32[n,3] on the GPU)."""
    n = int(points.shape[0])
    if out_obj is None:
        out_obj = torch.empty(n, dtype=torch.int32, device=points.device)
    if out_inside is None:
        out_inside = torch.empty(n, dtype=torch.uint8, device=points.device)
    fn = _lib.load().rs_pim_filtered if filtered else _lib.load().rs_pim
    _check(fn(bvh.handle, _ptr(points), n, float(direction[0]), float(direction[1]), float(direction[2]),
              _ptr(out_obj), _ptr(out_inside), _stream(stream)), "rs_pim")
    return out_obj, out_inside


def compact_hits(obj: torch.Tensor, stream=None) -> Tuple[torch.Tensor, torch.Tensor]:
    """(point ids, objects) of the points with obj != -1, in ascending point order."""
    n = int(obj.numel())
    ids = torch.empty(max(n, 1), dtype=torch.int32, device=obj.device)
    objs = torch.empty(max(n, 1), dtype=torch.int32, device=obj.device)
    cnt = ctypes.c_uint64()
    _check(_lib.load().rs_compact_hits(_ptr(obj), n, _ptr(ids), _ptr(objs), n, ctypes.byref(cnt), _stream(stream)),
           "rs_compact_hits")
    return ids[:cnt.value], objs[:cnt.value]


def extract_edges(V: torch.Tensor, I: torch.Tensor, T: torch.Tensor, stream=None):
    """Unique-edge payload (starts, ends, offsets, counts, sources) of device-resident
    triangles, identical to EdgePreprocessor::extractEdges
    (preprocess/src/EdgePreprocessor.cpp:41-119)."""
    nV, nF = int(V.shape[0]), int(I.shape[0])
    cap = max(3 * nF, 1)
    dev = V.device
    starts = torch.empty((cap, 3), dtype=torch.float32, device=dev)
    ends = torch.empty((cap, 3), dtype=torch.float32, device=dev)
    offsets = torch.empty(cap, dtype=torch.int32, device=dev)
    counts = torch.empty(cap, dtype=torch.int32, device=dev)
    sources = torch.empty(cap, dtype=torch.int32, device=dev)
    nE, nS = ctypes.c_uint64(), ctypes.c_uint64()
    _check(_lib.load().rs_extract_edges(_ptr(V), nV, _ptr(I), nF, _ptr(T), _ptr(starts), _ptr(ends), _ptr(offsets),
                                        _ptr(counts), _ptr(sources), cap, ctypes.byref(nE), ctypes.byref(nS),
                                        _stream(stream)), "rs_extract_edges")
    e, s = nE.value, nS.value
    return starts[:e], ends[:e], offsets[:e], counts[:e], sources[:s]


class PairSet:
    """Open-addressing table of pair keys (id1<<32 | id2)."""

    def __init__(self, capacity: int, pow2: bool = True, stream=None):
        h = ctypes.c_void_p()
        _check(_lib.load().rs_pairset_create(int(capacity), int(pow2), ctypes.byref(h), _stream(stream)),
               "rs_pairset_create")
        self.handle = h

    def clear(self, stream=None):
        _check(_lib.load().rs_pairset_clear(self.handle, _stream(stream)), "rs_pairset_clear")

    def set_edge_rule(self, max_hits: int = 100, next_float: bool = False):
        """Hit rule of the edge rays inserting into this table (rs_pairset_set_edge_rule):
        at most max_hits crossings per edge, the next searched from t + 1e-6, or from the
        next float after t when next_float."""
        _check(_lib.load().rs_pairset_set_edge_rule(self.handle, int(max_hits), int(next_float)),
               "rs_pairset_set_edge_rule")

    def info(self, stream=None):
        cap, cnt = ctypes.c_uint64(), ctypes.c_uint64()
        _check(_lib.load().rs_pairset_info(self.handle, ctypes.byref(cap), ctypes.byref(cnt), _stream(stream)),
               "rs_pairset_info")
        return cap.value, cnt.value

    def finalize(self, order: int = 0, stream=None) -> torch.Tensor:
        """Sorted unique keys as an int64 tensor on the GPU (bit pattern of the u64 keys),
        written in the order of `stream` (the current stream waits for it when they differ)."""
        _, cnt = self.info(stream)
        out = torch.empty(max(cnt, 1), dtype=torch.int64, device="cuda")
        n = ctypes.c_uint64()
        _check(_lib.load().rs_pairset_finalize(self.handle, int(order) | RS_FINALIZE_NO_WAIT, _ptr(out), cnt,
                                               ctypes.byref(n), _stream(stream)), "rs_pairset_finalize")
        if stream is not None and stream != torch.cuda.current_stream():
            torch.cuda.current_stream().wait_stream(stream)
        return out[:n.value]

    def close(self):
        if self.handle:
            _lib.load().rs_pairset_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def edge_join(target: Bvh, source: DeviceGeometry, ps: PairSet, swap: bool = False, stream=None) -> None:
    s, e, off, cnt, src = source.edge_ptrs()
    _check(_lib.load().rs_edge_join(target.handle, s, e, off, cnt, src, source.nE, int(swap), ps.handle,
                                    _stream(stream)), "rs_edge_join")


def containment(target: Bvh, source: DeviceGeometry, ps: PairSet, swap: bool = False, stream=None) -> None:
    _check(_lib.load().rs_containment(target.handle, _ptr(source.V), source.nV, _ptr(source.I), source.nF,
                                      _ptr(source.T), int(swap), ps.handle, _stream(stream)), "rs_containment")


def triangle_join(target: Bvh, source: DeviceGeometry, ps: PairSet, swap: bool = False, stream=None) -> None:
    """Legacy per-triangle overlap (mesh_overlap.cu:126-179): the source triangles' own edges
    traced against target, (source object, target object) keys, or swapped."""
    _check(_lib.load().rs_triangle_join(target.handle, _ptr(source.V), source.nV, _ptr(source.I), source.nF,
                                        _ptr(source.T), int(swap), ps.handle, _stream(stream)), "rs_triangle_join")


def edge_index(geom: "DeviceGeometry", out: Optional[torch.Tensor] = None, stream=None):
    """Slab index of a geometry's edge payload (rs_edge_index): an int64 tensor of
    3 + ceil(nE / 256) entries (on the GPU, or into `out`, e.g. pinned host memory) and
    whether the payload is in the reference's key order (else the index only disables
    itself)."""
    s, e, _, _, src = geom.edge_ptrs()
    n = 3 + (int(geom.nE) + 255) // 256
    if out is None:
        out = torch.empty(n, dtype=torch.int64, device="cuda")
    ordered = ctypes.c_int()
    _check(_lib.load().rs_edge_index(s, e, src, int(geom.nE), int(geom.edges[4].numel()), _kernel_ptr(out),
                                     ctypes.byref(ordered), _stream(stream)), "rs_edge_index")
    return out, bool(ordered.value)


def overlap_join(A: Bvh, B: Bvh, ps: PairSet, direction: int = 0, with_containment: bool = False,
                 stream=None, edges_ready=None, indexes=None) -> None:
    """Both edge directions (and containment when asked) into ps, growing it on overflow.
    edges_ready = (event for A's edges, event for B's edges) (torch.cuda.Event, either None):
    the broad phase runs at once, each direction's rays wait for their event.  indexes =
    (A's slab index, B's) from edge_index (either None): the live-edge check reads only the
    slabs of objects with partners (rs_overlap_join_indexed)."""
    ea = A.geom.edge_ptrs()
    eb = B.geom.edge_ptrs()
    L = _lib.load()
    if indexes is not None:
        evs = [ctypes.c_void_p(e.cuda_event) if e is not None else None for e in (edges_ready or (None, None))]
        ia, ib = (_kernel_ptr(t) for t in indexes)
        _check(L.rs_overlap_join_indexed(A.handle, *ea, A.geom.nE, ia, B.handle, *eb, B.geom.nE, ib, int(direction),
                                         int(with_containment), ps.handle, evs[0], evs[1], _stream(stream)),
               "rs_overlap_join_indexed")
        return
    if edges_ready is None:
        _check(L.rs_overlap_join(A.handle, *ea, A.geom.nE, B.handle, *eb, B.geom.nE, int(direction),
                                 int(with_containment), ps.handle, _stream(stream)), "rs_overlap_join")
        return
    evs = [ctypes.c_void_p(e.cuda_event) if e is not None else None for e in edges_ready]
    _check(L.rs_overlap_join_after(A.handle, *ea, A.geom.nE, B.handle, *eb, B.geom.nE, int(direction),
                                   int(with_containment), ps.handle, evs[0], evs[1], _stream(stream)),
           "rs_overlap_join_after")


def overlap_join_edges(A: Bvh, edges_a, B: Bvh, edges_b, ps: PairSet, stream=None) -> None:
    """rs_overlap_join (both directions, broad phase, table growth) with explicit edge
    payloads: edges_a = (starts, ends, offsets, counts, sources) device tensors of edges of
    A's objects -- any contiguous range of A's payload, its sources array whole -- traced
    against B, and edges_b likewise against A."""
    def ptrs(e):
        return [t.data_ptr() for t in e], int(e[0].shape[0])
    pa, na = ptrs(edges_a)
    pb, nb = ptrs(edges_b)
    _check(_lib.load().rs_overlap_join(A.handle, *pa, na, B.handle, *pb, nb, 0, 0, ps.handle, _stream(stream)),
           "rs_overlap_join")


def containment_range(target: Bvh, source: DeviceGeometry, tri_lo: int, tri_hi: int, ps: PairSet,
                      swap: bool = False, stream=None) -> None:
    """Containment rays of the source objects whose triangles are [tri_lo, tri_hi) (each
    object's triangles stored together, all of them inside the range)."""
    I = source.I[tri_lo:tri_hi]
    T = source.T[tri_lo:tri_hi]
    _check(_lib.load().rs_containment(target.handle, _ptr(source.V), source.nV, _ptr(I), int(tri_hi - tri_lo),
                                      _ptr(T), int(swap), ps.handle, _stream(stream)), "rs_containment")


def overlap_join_filtered(A: DeviceGeometry, B: DeviceGeometry, ps: PairSet, direction: int = 0,
                          with_containment: bool = False, leaf_size: int = 0, stream=None) -> None:
    """The join of overlap_join from the two geometries directly, with the BVHs built over
    the triangles of the objects whose boxes overlap the other set's (rs_overlap_join_filtered)."""
    ea, eb = A.edge_ptrs(), B.edge_ptrs()
    _check(_lib.load().rs_overlap_join_filtered(
        _ptr(A.V), A.nV, _ptr(A.I), A.nF, _ptr(A.T), *ea, A.nE, _ptr(B.V), B.nV, _ptr(B.I), B.nF, _ptr(B.T), *eb,
        B.nE, int(direction), int(with_containment), int(leaf_size), ps.handle, _stream(stream)),
        "rs_overlap_join_filtered")


def keys_to_pairs(keys) -> np.ndarray:
    """u64 keys (id1<<32 | id2) -> int32[n,2] (id1, id2)."""
    k = np.asarray(keys.cpu().numpy() if isinstance(keys, torch.Tensor) else keys).astype(np.uint64)
    return np.stack([(k >> np.uint64(32)).astype(np.int64), (k & np.uint64(0xffffffff)).astype(np.int64)],
                    axis=1).astype(np.int32)


def cell_volume(grid: Grid) -> float:
    """Cell volume from mesh1's grid bounds as raytracer_overlap_estimated_main.cpp:256-262 computes it."""
    f32 = np.float32
    w = f32(grid.max_bound[0]) - f32(grid.min_bound[0])
    h = f32(grid.max_bound[1]) - f32(grid.min_bound[1])
    d = f32(grid.max_bound[2]) - f32(grid.min_bound[2])
    cx = f32(w / f32(grid.resolution[0]))
    cy = f32(h / f32(grid.resolution[1]))
    cz = f32(d / f32(grid.resolution[2]))
    return float(f32(f32(cx * cy) * cz))


def estimate_grid(cellsA: torch.Tensor, cellsB: torch.Tensor, ncells: int, cell_vol: float, epsilon: float = 0.001,
                  gamma: float = 0.8, stream=None):
    raw = ctypes.c_double()
    means = (ctypes.c_float * 4)()
    _check(_lib.load().rs_estimate_grid(_ptr(cellsA), _ptr(cellsB), int(ncells), float(cell_vol), float(epsilon),
                                        float(gamma), ctypes.byref(raw), means, _stream(stream)), "rs_estimate_grid")
    return raw.value, list(means)


def estimate_pairs(A: DeviceGeometry, B: DeviceGeometry, epsilon: float = 0.001, gamma: float = 0.8,
                   alpha_correction: bool = True, stream=None) -> Tuple[int, float]:
    """Estimated pair count (0 when either set has no grid or the grids differ in size)."""
    ga, gb = A.host.grid, B.host.grid
    if ga is None or gb is None or A.cells is None or B.cells is None:
        return 0, 0.0
    ncells = int(ga.resolution[0]) * int(ga.resolution[1]) * int(ga.resolution[2])
    if len(ga.cells) != ncells or len(gb.cells) != ncells:
        return 0, 0.0
    cv = cell_volume(ga)
    raw, means = estimate_grid(A.cells, B.cells, ncells, cv, epsilon, gamma, stream)
    m = (ctypes.c_float * 4)(*means)
    est = _lib.load().rs_estimate_pairs_from_raw(raw, m, cv, int(alpha_correction))
    return int(est), raw


def hash_size_pow2(est: int) -> int:
    return int(_lib.load().rs_hash_size_pow2(int(est)))


def hash_size_odd(est: int, load_factor: float = 0.5) -> int:
    return int(_lib.load().rs_hash_size_odd(int(est), float(load_factor)))
