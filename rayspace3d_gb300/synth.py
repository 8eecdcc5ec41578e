"""Seeded synthetic datasets for the query path, written straight to ``.pre`` v2.

The reference builds its datasets offline (OBJ generators under ``scripts/`` and the
``preprocess_dataset`` tool); this module replaces that pipeline with numpy so the
benchmark and the tests can build the same kinds of inputs on any machine:

* icospheres of subdivision level L (V = 10*4^L+2, F = 20*4^L, E = 30*4^L unique edges),
  scaled, rotated by a Haar-uniform quaternion and translated;
* the unique-edge payload, restating ``EdgePreprocessor::extractEdges``
  (``preprocess/src/EdgePreprocessor.cpp:41-119``): endpoints quantised with
  ``llround(x*1e5)``, key = ordered pair of quantised endpoints in ``std::map`` order,
  endpoints taken from the first occurrence, source objects in first-seen order;
* grid statistics, restating ``generateGridStats``
  (``preprocess/src/preprocess_dataset.cpp:37-181``).  The reference visits its objects
  in the iteration order of a ``std::unordered_map<int, ObjectStats>`` and sums floats
  per cell in that order; ``unordered_map_order`` reproduces GCC libstdc++'s order, so
  the per-cell means match the reference built with GCC bit for bit.
"""
from __future__ import annotations

from typing import List, Optional, Tuple

import numpy as np

from .formats import Edges, Geometry, Grid, GRID_CELL_DTYPE

_ICO_CACHE = {}


def icosphere(level: int) -> Tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: float64 vertices on the unit sphere and uint32 triangles
    (counter-clockwise seen from outside).  Subdivision splits every triangle into four
    through its edge midpoints, projected back onto the sphere."""
    if level in _ICO_CACHE:
        return _ICO_CACHE[level]
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    for _ in range(level):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mids = V[uniq[:, 0]] + V[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(V)
        V = np.concatenate([V, mids])
        nf = len(F)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        F = np.concatenate([np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
                            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    out = (V, F.astype(np.uint32))
    _ICO_CACHE[level] = out
    return out


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Haar-uniform rotations from normalised Gaussian quaternions, float64[n,3,3]."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def assemble(levels: np.ndarray, radii: np.ndarray, rots: Optional[np.ndarray],
             centers: np.ndarray) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Concatenate transformed icospheres into one triangle soup with per-object
    vertex blocks.  Returns float32 V[N,3], uint32 I[F,3], int32 tri2obj[F]."""
    Vs: List[np.ndarray] = []
    Is: List[np.ndarray] = []
    Ts: List[np.ndarray] = []
    voff = 0
    levels = np.asarray(levels)
    for lvl in np.unique(levels):
        pass
    for i in range(len(levels)):
        v, f = icosphere(int(levels[i]))
        p = v * radii[i]
        if rots is not None:
            p = p @ rots[i].T
        p = p + centers[i]
        Vs.append(p.astype(np.float32))
        Is.append(f + np.uint32(voff))
        Ts.append(np.full(len(f), i, dtype=np.int32))
        voff += len(v)
    return np.concatenate(Vs), np.concatenate(Is).astype(np.uint32), np.concatenate(Ts)


def assemble_uniform(level: int, radii: np.ndarray, rots: Optional[np.ndarray],
                     centers: np.ndarray) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Vectorised ``assemble`` for objects that all share one subdivision level."""
    v, f = icosphere(level)
    n = len(radii)
    p = v[None, :, :] * np.asarray(radii, dtype=np.float64)[:, None, None]
    if rots is not None:
        p = np.einsum("nvk,njk->nvj", p, rots)
    p = p + np.asarray(centers, dtype=np.float64)[:, None, :]
    V = p.astype(np.float32).reshape(-1, 3)
    I = (f[None, :, :].astype(np.int64) + (np.arange(n, dtype=np.int64) * len(v))[:, None, None])
    I = I.reshape(-1, 3).astype(np.uint32)
    T = np.repeat(np.arange(n, dtype=np.int32), len(f))
    return V, I, T


def _llround(x: np.ndarray) -> np.ndarray:
    """C ``llround``: round half away from zero, exactly."""
    r = np.trunc(x)
    frac = x - r
    up = np.abs(frac) >= 0.5
    return (r + np.where(up, np.sign(x), 0.0)).astype(np.int64)


def extract_edges(V: np.ndarray, I: np.ndarray, T: np.ndarray) -> Edges:
    """Unique-edge payload exactly as EdgePreprocessor::extractEdges builds it."""
    V = np.asarray(V, dtype=np.float32)
    I = np.asarray(I, dtype=np.int64)
    T = np.asarray(T, dtype=np.int32)
    nF = len(I)
    if nF == 0 or len(V) == 0:
        z = np.zeros((0, 3), np.float32)
        zi = np.zeros(0, np.int32)
        return Edges(z, z.copy(), zi, zi.copy(), zi.copy())
    valid = (I < len(V)).all(axis=1)
    tri = np.nonzero(valid)[0]
    # Triangle-major, edge-minor order: (v0,v1), (v1,v2), (v2,v0).
    a = I[tri][:, [0, 1, 2]].reshape(-1)
    b = I[tri][:, [1, 2, 0]].reshape(-1)
    obj = np.repeat(T[tri], 3)
    pa = V[a]
    pb = V[b]
    qa = _llround(pa.astype(np.float64) * 1e5)
    qb = _llround(pb.astype(np.float64) * 1e5)
    # q1 < q0 lexicographically -> swap (key only)
    less = (qb[:, 0] < qa[:, 0]) | ((qb[:, 0] == qa[:, 0]) & (
        (qb[:, 1] < qa[:, 1]) | ((qb[:, 1] == qa[:, 1]) & (qb[:, 2] < qa[:, 2]))))
    k0 = np.where(less[:, None], qb, qa)
    k1 = np.where(less[:, None], qa, qb)
    m = len(a)
    pos = np.arange(m, dtype=np.int64)
    order = np.lexsort((pos, k1[:, 2], k1[:, 1], k1[:, 0], k0[:, 2], k0[:, 1], k0[:, 0]))
    ks = np.concatenate([k0, k1], axis=1)[order]
    newgrp = np.ones(m, dtype=bool)
    newgrp[1:] = (ks[1:] != ks[:-1]).any(axis=1)
    gid_sorted = np.cumsum(newgrp) - 1
    ngroups = int(gid_sorted[-1]) + 1
    first_pos = order[newgrp]                      # earliest occurrence of each key
    starts = pa[first_pos]
    ends = pb[first_pos]
    # Source objects: unique (group, obj) pairs, kept in first-seen order.
    gid = np.empty(m, dtype=np.int64)
    gid[order] = gid_sorted
    o2 = np.lexsort((pos, obj, gid))
    g_o = gid[o2]
    ob_o = obj[o2]
    keep = np.ones(m, dtype=bool)
    keep[1:] = (g_o[1:] != g_o[:-1]) | (ob_o[1:] != ob_o[:-1])
    sel = o2[keep]                                  # first position of each (group,obj)
    o3 = np.lexsort((pos[sel], gid[sel]))
    sel = sel[o3]
    sources = obj[sel].astype(np.int32)
    counts = np.bincount(gid[sel], minlength=ngroups).astype(np.int32)
    offsets = np.zeros(ngroups, dtype=np.int64)
    offsets[1:] = np.cumsum(counts)[:-1]
    return Edges(starts.astype(np.float32), ends.astype(np.float32), offsets.astype(np.int32),
                 counts, sources)


# Bucket counts a libstdc++ std::unordered_map<int, V> passes through when keys are inserted
# one at a time (max_load_factor 1): the table rehashes when the (count+1)-th key arrives.
_UMAP_BUCKETS = (13, 29, 59, 127, 257, 541, 1109, 2357, 5087, 10273, 20753, 42043, 85229, 172933, 351061,
                 712697, 1447153, 2938679, 5967347, 12117689, 24607243, 49969847)


def unordered_map_order(keys) -> List[int]:
    """Iteration order of a GCC ``std::unordered_map<int, V>`` after ``m[k]`` for each key
    in turn (repeated keys ignored).  Model: one singly linked node list; a key whose
    bucket is empty goes to the front of the list, otherwise to the front of its bucket's
    run; a rehash walks the list front to back and re-inserts by the same rule, which
    reverses the runs.  std::hash<int> is the identity (sign-extended to 64 bits)."""
    BB = "head"
    nxt = {BB: None}
    buckets = {}          # bucket -> node before the bucket's first node
    nb = 1
    growth = iter(_UMAP_BUCKETS)
    count = 0
    for k in keys:
        k = int(k)
        if k in nxt:
            continue
        if count + 1 > (nb if count else 0):
            try:
                nb = next(growth)
            except StopIteration:
                raise ValueError("too many objects for the unordered_map order model") from None
            p, nxt[BB], buckets, before = nxt[BB], None, {}, None
            while p is not None:
                after, b = nxt[p], (p & 0xFFFFFFFFFFFFFFFF) % nb
                if b not in buckets:
                    nxt[p], nxt[BB], buckets[b] = nxt[BB], p, BB
                    if nxt[p] is not None:
                        buckets[before] = p
                    before = b
                else:
                    nxt[p], nxt[buckets[b]] = nxt[buckets[b]], p
                p = after
        b = (k & 0xFFFFFFFFFFFFFFFF) % nb
        if b in buckets:
            nxt[k], nxt[buckets[b]] = nxt[buckets[b]], k
        else:
            nxt[k], nxt[BB] = nxt[BB], k
            if nxt[k] is not None:
                buckets[(nxt[k] & 0xFFFFFFFFFFFFFFFF) % nb] = k
            buckets[b] = BB
        count += 1
    out, p = [], nxt[BB]
    while p is not None:
        out.append(p)
        p = nxt[p]
    return out


def grid_stats(V: np.ndarray, I: np.ndarray, T: np.ndarray, resolution: int = 128,
               world_size: float = -1.0) -> Grid:
    """Per-cell statistics as generateGridStats computes them (float32 arithmetic)."""
    f32 = np.float32
    V = np.asarray(V, dtype=np.float32)
    I = np.asarray(I, dtype=np.int64)
    T = np.asarray(T, dtype=np.int64)
    R = int(resolution)
    if world_size <= 0:
        mn = V.min(axis=0) if len(V) else np.full(3, 1e30, f32)
        mx = V.max(axis=0) if len(V) else np.full(3, -1e30, f32)
    else:
        mn = np.zeros(3, f32)
        mx = np.full(3, world_size, f32)
    mn = mn.astype(f32)
    mx = mx.astype(f32)
    rng_ = (mx - mn).astype(f32)
    cs = (rng_ / f32(R)).astype(f32)
    cells = np.zeros(R * R * R, dtype=GRID_CELL_DTYPE)
    valid = (I < len(V)).all(axis=1)
    I = I[valid]
    T = T[valid]
    if len(I) == 0:
        return Grid(mn, mx, np.array([R, R, R], np.uint32), cells)
    objs, first, tinv = np.unique(T, return_index=True, return_inverse=True)
    nobj = len(objs)
    v0, v1, v2 = V[I[:, 0]], V[I[:, 1]], V[I[:, 2]]
    tmin = np.minimum(np.minimum(v0, v1), v2)
    tmax = np.maximum(np.maximum(v0, v1), v2)
    omin = np.full((nobj, 3), f32(1e30), f32)
    omax = np.full((nobj, 3), f32(-1e30), f32)
    np.minimum.at(omin, tinv, tmin)
    np.maximum.at(omax, tinv, tmax)
    center = ((omin + omax) * f32(0.5)).astype(f32)
    c = center[tinv]
    t0, t1, t2 = (v0 - c).astype(f32), (v1 - c).astype(f32), (v2 - c).astype(f32)
    cx = (t0[:, 1] * t1[:, 2] - t0[:, 2] * t1[:, 1]).astype(f32)
    cy = (t0[:, 2] * t1[:, 0] - t0[:, 0] * t1[:, 2]).astype(f32)
    cz = (t0[:, 0] * t1[:, 1] - t0[:, 1] * t1[:, 0]).astype(f32)
    sv = ((cx * t2[:, 0] + cy * t2[:, 1]) + cz * t2[:, 2]).astype(f32)
    vol = np.zeros(nobj, dtype=np.float64)
    np.add.at(vol, tinv, sv.astype(np.float64))     # double accumulation in triangle order
    meshvol = (np.abs(vol.astype(f32)) / f32(6.0)).astype(f32)
    w = (omax - omin).astype(f32)
    aabb = ((w[:, 0] * w[:, 1]) * w[:, 2]).astype(f32)
    aabb = np.where(aabb < f32(1e-9), f32(1e-9), aabb).astype(f32)
    ratio = (meshvol / aabb).astype(f32)
    ratio = np.where(ratio > f32(1.0), f32(1.0), ratio).astype(f32)
    ctr = ((omin + omax) * f32(0.5)).astype(f32)
    avg = (((w[:, 0] + w[:, 1]) + w[:, 2]) / f32(3.0)).astype(f32)
    anchor = ((ctr - mn) / cs).astype(f32)
    ai = np.trunc(anchor).astype(np.int64)
    inb = ((ai >= 0) & (ai < R)).all(axis=1)
    aidx = (ai[:, 2] * R + ai[:, 1]) * R + ai[:, 0]
    np.add.at(cells["CenterCount"], aidx[inb], np.uint32(1))
    lo = np.maximum(0, np.trunc(((omin - mn) / cs).astype(f32)).astype(np.int64))
    hi = np.minimum(R - 1, np.trunc((((omax - mn) - f32(1e-5)) / cs).astype(f32)).astype(np.int64))
    touch = np.zeros(R * R * R, np.uint32)
    asum = np.zeros(R * R * R, np.float32)
    rsum = np.zeros(R * R * R, np.float32)
    visit = np.searchsorted(objs, unordered_map_order(objs[np.argsort(first, kind="stable")]))
    for o in visit:         # the reference's object order; float32 accumulation per cell
        x0, y0, z0 = lo[o]
        x1, y1, z1 = hi[o]
        if x1 < x0 or y1 < y0 or z1 < z0:
            continue
        zz, yy, xx = np.meshgrid(np.arange(z0, z1 + 1), np.arange(y0, y1 + 1), np.arange(x0, x1 + 1),
                                 indexing="ij")
        idx = ((zz * R + yy) * R + xx).reshape(-1)
        touch[idx] += np.uint32(1)
        asum[idx] = (asum[idx] + avg[o]).astype(f32)
        rsum[idx] = (rsum[idx] + ratio[o]).astype(f32)
    nz = touch > 0
    cells["TouchCount"] = touch
    cells["AvgSizeMean"] = np.where(nz, asum / np.maximum(touch, 1).astype(f32), f32(0)).astype(f32)
    cells["VolRatio"] = np.where(nz, rsum / np.maximum(touch, 1).astype(f32), f32(0)).astype(f32)
    return Grid(mn, mx, np.array([R, R, R], np.uint32), cells)


def make_geometry(V, I, T, edges: bool = True, grid_resolution: int = 0,
                  world_size: float = -1.0) -> Geometry:
    g = Geometry(np.asarray(V, np.float32), np.asarray(I, np.uint32), np.asarray(T, np.int32),
                 total_triangles=len(I))
    if edges:
        g.edges = extract_edges(V, I, T)
    if grid_resolution > 0:
        g.grid = grid_stats(V, I, T, grid_resolution, world_size)
    return g


# --- workloads -------------------------------------------------------------------------

def pim_workload(n_points: int = 1_000_000, level: int = 4, seed: int = 0,
                 extent: float = 1.5) -> Tuple[Geometry, np.ndarray]:
    """One closed unit icosphere at the origin and points uniform in [-extent, extent]^3."""
    v, f = icosphere(level)
    g = Geometry(v.astype(np.float32), f.copy(), np.zeros(len(f), np.int32), total_triangles=len(f))
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-extent, extent, size=(n_points, 3)).astype(np.float32)
    return g, pts


def sphere_set(n_objects: int, level: int, r_lo: float, r_hi: float, world: float,
               rng: np.random.Generator, edges: bool = True, grid_resolution: int = 0,
               grid_world: Optional[float] = None) -> Geometry:
    """n icospheres of one level, radius log-uniform in [r_lo, r_hi], Haar rotation,
    centre uniform in [0, world]^3."""
    radii = np.exp(rng.uniform(np.log(r_lo), np.log(r_hi), n_objects))
    rots = random_rotations(rng, n_objects)
    centers = rng.uniform(0.0, world, size=(n_objects, 3))
    V, I, T = assemble_uniform(level, radii, rots, centers)
    return make_geometry(V, I, T, edges=edges, grid_resolution=grid_resolution,
                         world_size=(world if grid_world is None else grid_world))


def overlap_workload(n_objects: int = 10_000, level: int = 2, world: float = 1000.0, seed: int = 1,
                     grid_resolution: int = 0) -> Tuple[Geometry, Geometry]:
    """Two sets of level-2 icospheres, radius log-uniform in [0.5, 2], uniform rotation,
    translation uniform in [0, world]^3.  Set A uses stream 1 of the seed, set B stream 2."""
    ss = np.random.SeedSequence(seed)
    ra, rb = [np.random.default_rng(s) for s in ss.spawn(2)]
    A = sphere_set(n_objects, level, 0.5, 2.0, world, ra, grid_resolution=grid_resolution)
    B = sphere_set(n_objects, level, 0.5, 2.0, world, rb, grid_resolution=grid_resolution)
    return A, B


def mixed_level_set(n_objects: int, levels: np.ndarray, r_lo: float, r_hi: float, world: float,
                    rng: np.random.Generator, inside_of: Optional[Tuple[np.ndarray, np.ndarray]] = None,
                    inside_frac: float = 0.0, grid_resolution: int = 0) -> Geometry:
    """Icospheres of uneven levels.  With ``inside_of=(centers, radii)`` a fraction of the
    objects is placed strictly inside a random object of the other set (scaled to at most
    half its radius, centre offset below 0.9*(R-r))."""
    radii = np.exp(rng.uniform(np.log(r_lo), np.log(r_hi), n_objects))
    rots = random_rotations(rng, n_objects)
    centers = rng.uniform(0.0, world, size=(n_objects, 3))
    if inside_of is not None and inside_frac > 0:
        oc, orad = inside_of
        k = int(round(inside_frac * n_objects))
        who = rng.choice(n_objects, size=k, replace=False)
        host = rng.integers(0, len(oc), size=k)
        # icosphere faces are inset from the sphere by at most 1-cos(edge angle); a level-1
        # host still contains a ball of radius 0.79*R, so stay well inside it.
        r_in = orad[host] * rng.uniform(0.1, 0.5, size=k) * 0.75
        room = np.maximum(orad[host] * 0.75 - r_in, 0.0) * 0.9
        dirn = rng.standard_normal((k, 3))
        dirn /= np.linalg.norm(dirn, axis=1, keepdims=True)
        off = dirn * (room * rng.uniform(0.0, 1.0, size=k) ** (1 / 3))[:, None]
        radii[who] = r_in
        centers[who] = oc[host] + off
    V, I, T = assemble(levels, radii, rots, centers)
    g = make_geometry(V, I, T, edges=True, grid_resolution=grid_resolution, world_size=world)
    g._centers = centers  # type: ignore[attr-defined]
    g._radii = radii      # type: ignore[attr-defined]
    return g


# --- degeneracy-heavy inputs ------------------------------------------------------------

_CUBE_F = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                    [3, 6, 2], [3, 7, 6], [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5]], dtype=np.uint32)


def cube_mesh(lo, hi) -> Tuple[np.ndarray, np.ndarray]:
    """Axis-aligned box as 8 vertices and 12 outward-wound triangles."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    V = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float32)
    return V, _CUBE_F.copy()


def box_set(boxes, edges: bool = True, grid_resolution: int = 0) -> Geometry:
    """One object per axis-aligned box (lo, hi), in the given order (grid statistics over the
    vertices' bounds when grid_resolution > 0)."""
    Vs, Is, Ts = [], [], []
    for k, (lo, hi) in enumerate(boxes):
        V, F = cube_mesh(lo, hi)
        Is.append(F + 8 * k)
        Vs.append(V)
        Ts.append(np.full(len(F), k, np.int32))
    return make_geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts), edges=edges,
                         grid_resolution=grid_resolution)


def cube_grid(nx: int, ny: int, nz: int, size: float = 1.0, origin=(0.0, 0.0, 0.0), edges: bool = True,
              grid_resolution: int = 0) -> Geometry:
    """nx*ny*nz unit cubes that share faces with their neighbours, one object each."""
    Vs, Is, Ts = [], [], []
    k = 0
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                lo = (origin[0] + x * size, origin[1] + y * size, origin[2] + z * size)
                hi = (lo[0] + size, lo[1] + size, lo[2] + size)
                v, f = cube_mesh(lo, hi)
                Vs.append(v)
                Is.append(f + np.uint32(8 * k))
                Ts.append(np.full(12, k, np.int32))
                k += 1
    return make_geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts), edges=edges,
                         grid_resolution=grid_resolution)


def snapped_points(g: Geometry, n: int, rng: np.random.Generator, frac_snapped: float = 0.2,
                   pad: float = 0.25) -> np.ndarray:
    """Points uniform in the padded bounds of g; a fraction is placed exactly on mesh
    vertices, on edges (convex combinations rounded to float32) and on faces."""
    V = np.asarray(g.vertices, np.float32)
    I = np.asarray(g.indices, np.int64)
    lo = V.min(axis=0) - pad
    hi = V.max(axis=0) + pad
    pts = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    k = int(n * frac_snapped)
    which = rng.integers(0, 3, size=k)
    tri = I[rng.integers(0, len(I), size=k)]
    a, b, c = V[tri[:, 0]], V[tri[:, 1]], V[tri[:, 2]]
    w = rng.uniform(0, 1, size=(k, 1))
    u = rng.dirichlet([1, 1, 1], size=k)
    snap = np.where(which[:, None] == 0, a,
                    np.where(which[:, None] == 1, (a + w * (b - a)),
                             u[:, :1] * a + u[:, 1:2] * b + u[:, 2:] * c)).astype(np.float32)
    idx = rng.choice(n, size=k, replace=False)
    pts[idx] = snap
    return pts
