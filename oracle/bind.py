"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and the cpu_baseline / reference leg of
``bench.py`` may import this module.  It builds ``oracle/_build/liboracle.so`` from
``oracle/oracle.cpp`` on first use if the library is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "liboracle.so")

_lib = None


def build_cmd():
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
            "-o", LIB_PATH, os.path.join(HERE, "oracle.cpp")]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        os.makedirs(LIB_DIR, exist_ok=True)
        subprocess.run(build_cmd(), check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        U64 = ctypes.c_uint64
        F = ctypes.c_float
        I = ctypes.c_int
        L.orc_pim.argtypes = [P, U64, P, U64, P, P, U64, F, F, F, P, I, I]
        L.orc_pim_filtered.argtypes = L.orc_pim.argtypes
        L.orc_edge_join.argtypes = [P, P, P, P, P, U64, P, U64, P, U64, P, I,
                                    ctypes.POINTER(ctypes.POINTER(U64)), ctypes.POINTER(U64), I, I, I, I]
        L.orc_containment.argtypes = [P, U64, P, U64, P, P, U64, P, U64, P, I,
                                      ctypes.POINTER(ctypes.POINTER(U64)), ctypes.POINTER(U64), I, I]
        L.orc_containment_diag.argtypes = [P, U64, P, U64, P, P, U64, P, U64, P, P, U64,
                                           ctypes.POINTER(ctypes.POINTER(U64)),
                                           ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32)), ctypes.POINTER(U64), I]
        L.orc_estimate_raw.argtypes = [P, P, U64, F, F, F]
        L.orc_estimate_raw.restype = ctypes.c_double
        L.orc_estimate_pairs.argtypes = [P, P, U64, P, P, P, F, F, I, ctypes.POINTER(ctypes.c_double)]
        L.orc_estimate_pairs.restype = ctypes.c_int64
        L.orc_orient.argtypes = [P, P, P, P]
        L.orc_perturbed_sign.argtypes = [P, P, P, P]
        L.orc_free.argtypes = [P]
        L.orc_segment_hits.argtypes = [P, P, P, U64, P, U64, P, P, P, U64, ctypes.POINTER(U64)]
        L.orc_box_mesh.argtypes = [P, U64, P, P]
        PF, PI = ctypes.POINTER(ctypes.POINTER(F)), ctypes.POINTER(ctypes.POINTER(ctypes.c_int32))
        L.orc_extract_edges.argtypes = [P, U64, P, U64, P, PF, PF, PI, PI, PI, ctypes.POINTER(U64),
                                        ctypes.POINTER(U64)]
        L.orc_grid_stats.argtypes = [P, U64, P, U64, P, I, F, P, P]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def pim(V, I, T, pts, direction=(0.0, 0.0, 1.0), threads=None, use_bvh=True, filtered=False):
    """Object id of the first counted hit for points inside (odd parity), else -1."""
    V, I, T, pts = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32), _c(pts, np.float32)
    out = np.empty(len(pts), dtype=np.int32)
    fn = lib().orc_pim_filtered if filtered else lib().orc_pim
    fn(_p(V), len(V), _p(I), len(I), _p(T), _p(pts), len(pts), float(direction[0]),
       float(direction[1]), float(direction[2]), _p(out), threads or os.cpu_count(), int(use_bvh))
    return out


def _take_keys(kp, nk):
    n = int(nk.value)
    out = np.ctypeslib.as_array(kp, shape=(max(n, 1),))[:n].copy() if n else np.zeros(0, np.uint64)
    lib().orc_free(ctypes.cast(kp, ctypes.c_void_p))
    return out


def edge_join(edges, V, I, T, swap=False, threads=None, use_bvh=True, max_hits=100, next_float=False):
    """Sorted unique pair keys (id1<<32|id2) of one edge-ray direction, each edge's crossings
    taken by the reference's edge loop (at most max_hits; t_min + 1e-6, or the next float)."""
    s, e = _c(edges.starts, np.float32), _c(edges.ends, np.float32)
    off, cnt, src = _c(edges.offsets, np.int32), _c(edges.counts, np.int32), _c(edges.sources, np.int32)
    V, I, T = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32)
    kp = ctypes.POINTER(ctypes.c_uint64)()
    nk = ctypes.c_uint64()
    lib().orc_edge_join(_p(s), _p(e), _p(off), _p(cnt), _p(src), len(s), _p(V), len(V), _p(I), len(I), _p(T),
                        int(swap), ctypes.byref(kp), ctypes.byref(nk), threads or os.cpu_count(), int(use_bvh),
                        int(max_hits), int(next_float))
    return _take_keys(kp, nk)


def segment_hits(start, end, V, I, T, cap=4096):
    """(t float32[], triangle uint64[]) of every crossing of one segment, unsorted."""
    st, en = _c(start, np.float32), _c(end, np.float32)
    V, I, T = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32)
    t = np.zeros(cap, np.float32)
    tri = np.zeros(cap, np.uint64)
    n = ctypes.c_uint64()
    lib().orc_segment_hits(_p(st), _p(en), _p(V), len(V), _p(I), len(I), _p(T), _p(t), _p(tri), cap, ctypes.byref(n))
    k = int(n.value)
    assert k <= cap, "more crossings than cap"
    return t[:k], tri[:k]


def containment(src_geom, V, I, T, swap=False, threads=None, use_bvh=True):
    sV, sI, sT = _c(src_geom.vertices, np.float32), _c(src_geom.indices, np.uint32), _c(src_geom.tri2obj, np.int32)
    V, I, T = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32)
    kp = ctypes.POINTER(ctypes.c_uint64)()
    nk = ctypes.c_uint64()
    lib().orc_containment(_p(sV), len(sV), _p(sI), len(sI), _p(sT), _p(V), len(V), _p(I), len(I), _p(T),
                          int(swap), ctypes.byref(kp), ctypes.byref(nk), threads or os.cpu_count(), int(use_bvh))
    return _take_keys(kp, nk)


def containment_diag(src_geom, V, I, T, threads=None):
    """(candidates[nObj], odd keys (src<<32|tgt) sorted, crossed-triangle count per key)."""
    sV, sI, sT = _c(src_geom.vertices, np.float32), _c(src_geom.indices, np.uint32), _c(src_geom.tri2obj, np.int32)
    V, I, T = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32)
    n_obj = int(sT.max()) + 1 if len(sT) else 0
    cand = np.zeros(max(n_obj, 1), np.uint32)
    kp = ctypes.POINTER(ctypes.c_uint64)()
    hp = ctypes.POINTER(ctypes.c_uint32)()
    nk = ctypes.c_uint64()
    rc = lib().orc_containment_diag(_p(sV), len(sV), _p(sI), len(sI), _p(sT), _p(V), len(V), _p(I), len(I), _p(T),
                                    _p(cand), len(cand), ctypes.byref(kp), ctypes.byref(hp), ctypes.byref(nk),
                                    threads or os.cpu_count())
    assert rc == 0
    n = int(nk.value)
    hits = np.ctypeslib.as_array(hp, shape=(max(n, 1),))[:n].copy() if n else np.zeros(0, np.uint32)
    lib().orc_free(ctypes.cast(hp, ctypes.c_void_p))
    return cand[:n_obj], _take_keys(kp, nk), hits


def overlap_join(A, B, threads=None, use_bvh=True, max_hits=100, next_float=False):
    """Union of both edge directions: A-edges into B, B-edges into A (swapped)."""
    k1 = edge_join(A.edges, B.vertices, B.indices, B.tri2obj, swap=False, threads=threads, use_bvh=use_bvh,
                   max_hits=max_hits, next_float=next_float)
    k2 = edge_join(B.edges, A.vertices, A.indices, A.tri2obj, swap=True, threads=threads, use_bvh=use_bvh,
                   max_hits=max_hits, next_float=next_float)
    return np.union1d(k1, k2).astype(np.uint64)


def intersection_join(A, B, threads=None, use_bvh=True, max_hits=100):
    """Overlap of both directions plus containment of both directions (sorted unique)."""
    parts = [overlap_join(A, B, threads, use_bvh, max_hits=max_hits),
             containment(A, B.vertices, B.indices, B.tri2obj, swap=False, threads=threads, use_bvh=use_bvh),
             containment(B, A.vertices, A.indices, A.tri2obj, swap=True, threads=threads, use_bvh=use_bvh)]
    return np.unique(np.concatenate(parts)).astype(np.uint64)


def estimate_raw(cellsA, cellsB, cell_volume, epsilon=0.001, gamma=0.8):
    a = np.ascontiguousarray(cellsA)
    b = np.ascontiguousarray(cellsB)
    return lib().orc_estimate_raw(_p(a), _p(b), len(a), cell_volume, epsilon, gamma)


def estimate_pairs(gridA, gridB, epsilon=0.001, gamma=0.8, alpha_correction=True):
    a = np.ascontiguousarray(gridA.cells)
    b = np.ascontiguousarray(gridB.cells)
    mn = _c(gridA.min_bound, np.float32)
    mx = _c(gridA.max_bound, np.float32)
    rs = _c(gridA.resolution, np.uint32)
    raw = ctypes.c_double()
    est = lib().orc_estimate_pairs(_p(a), _p(b), len(a), _p(mn), _p(mx), _p(rs), epsilon, gamma,
                                   int(alpha_correction), ctypes.byref(raw))
    return int(est), float(raw.value)


def orient(d, o, a, b):
    arrs = [_c(x, np.float32) for x in (d, o, a, b)]
    return lib().orc_orient(*[_p(x) for x in arrs])


def perturbed_sign(d, o, a, b):
    arrs = [_c(x, np.float32) for x in (d, o, a, b)]
    return lib().orc_perturbed_sign(*[_p(x) for x in arrs])


def box_mesh(V):
    V = _c(V, np.float32)
    bv = np.empty((8, 3), np.float32)
    bi = np.empty((12, 3), np.uint32)
    lib().orc_box_mesh(_p(V), len(V), _p(bv), _p(bi))
    return bv, bi


def containment_strict(A, B, threads=None, use_bvh=True):
    """raytracer_containment: B objects inside A objects (B->A containment rays, as (a, b))
    whose pair is not an overlap pair.  Returns (strict containment keys, overlap keys)."""
    overlap = overlap_join(A, B, threads, use_bvh, max_hits=256, next_float=True)  # mesh_containment.cu:99-170
    inside = containment(B, A.vertices, A.indices, A.tri2obj, swap=True, threads=threads, use_bvh=use_bvh)
    return np.setdiff1d(inside, overlap).astype(np.uint64), overlap


def extract_edges(V, I, T):
    """(starts, ends, offsets, counts, sources) of EdgePreprocessor::extractEdges."""
    V, I, T = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32)
    L = lib()
    ptr_f = [ctypes.POINTER(ctypes.c_float)() for _ in range(2)]
    ptr_i = [ctypes.POINTER(ctypes.c_int32)() for _ in range(3)]
    ne, ns = ctypes.c_uint64(), ctypes.c_uint64()
    L.orc_extract_edges(_p(V), len(V), _p(I), len(I), _p(T), ctypes.byref(ptr_f[0]), ctypes.byref(ptr_f[1]),
                        ctypes.byref(ptr_i[0]), ctypes.byref(ptr_i[1]), ctypes.byref(ptr_i[2]), ctypes.byref(ne),
                        ctypes.byref(ns))
    n_e, n_s = ne.value, ns.value
    out = [np.ctypeslib.as_array(ptr_f[0], shape=(max(n_e, 1) * 3,))[:3 * n_e].reshape(-1, 3).copy(),
           np.ctypeslib.as_array(ptr_f[1], shape=(max(n_e, 1) * 3,))[:3 * n_e].reshape(-1, 3).copy(),
           np.ctypeslib.as_array(ptr_i[0], shape=(max(n_e, 1),))[:n_e].copy(),
           np.ctypeslib.as_array(ptr_i[1], shape=(max(n_e, 1),))[:n_e].copy(),
           np.ctypeslib.as_array(ptr_i[2], shape=(max(n_s, 1),))[:n_s].copy()]
    for p in ptr_f + ptr_i:
        L.orc_free(ctypes.cast(p, ctypes.c_void_p))
    return out


def grid_stats(V, I, T, res, world_size):
    """(bounds float32[6], cells uint8[res^3 * 16]) of generateGridStats."""
    V, I, T = _c(V, np.float32), _c(I, np.uint32), _c(T, np.int32)
    cells = np.zeros(int(res) ** 3 * 16, np.uint8)
    b = np.zeros(6, np.float32)
    lib().orc_grid_stats(_p(V), len(V), _p(I), len(I), _p(T), int(res), float(world_size), _p(cells), _p(b))
    return b, cells
