"""Seeded synthetic workloads generated directly in device memory (torch on the GPU).

For workloads too large to build on the host (the batched configuration: hundreds of
millions of points and triangles): instanced icospheres and boxes with per-object
transforms, their edge payloads, and query points with a share snapped exactly onto
mesh vertices, edges and faces.  Instances of one template never share quantised
edge endpoints (random transforms), so each object's unique template edges are its
edge payload with the object as the only source -- the set that
``EdgePreprocessor::extractEdges`` (preprocess/src/EdgePreprocessor.cpp:41-119) would
produce, with its first-occurrence orientation, listed per object rather than in
``std::map`` order.  Edge-ray results do not depend on the order.  Face-sharing cube
blocks, whose edges are shared across objects, come from the host generator
(``synth.cube_grid``) instead.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import torch

from . import synth
from .api import DeviceGeometry

_TEMPLATE = {}


def _template(kind: str, level: int, device):
    key = (kind, level, str(device))
    if key not in _TEMPLATE:
        if kind == "sphere":
            v, f = synth.icosphere(level)
        else:
            v, f = synth.cube_mesh((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))
            v = v.astype(np.float64)
        # Edges in face order (v0v1, v1v2, v2v0 of each face), each kept with the
        # orientation of its first occurrence, as the reference's extraction does.
        e = np.stack([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=1).reshape(-1, 2).astype(np.int64)
        _, first = np.unique(np.sort(e, axis=1), axis=0, return_index=True)
        e = e[np.sort(first)]
        _TEMPLATE[key] = (torch.from_numpy(np.asarray(v, np.float64)).to(device),
                          torch.from_numpy(np.asarray(f, np.int64)).to(device),
                          torch.from_numpy(e).to(device))
    return _TEMPLATE[key]


def _rotations(g: torch.Generator, n: int, device) -> torch.Tensor:
    q = torch.randn((n, 4), generator=g, device=device, dtype=torch.float64)
    q = q / q.norm(dim=1, keepdim=True)
    w, x, y, z = q.unbind(1)
    R = torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                     2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                     2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], dim=1)
    return R.view(n, 3, 3)


def instanced_set(n_objects: int, level: int, r_lo: float, r_hi: float, world: float, seed: int,
                  kind: str = "sphere", device="cuda", centers: Optional[torch.Tensor] = None) -> DeviceGeometry:
    """n objects of one template (icosphere of `level`, or a box), radius log-uniform in
    [r_lo, r_hi], Haar rotation, centre uniform in [0, world]^3 (or the given float64
    centers[n,3]); with edges."""
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    tv, tf, te = _template(kind, level, dev)
    nv, nf, ne = tv.shape[0], tf.shape[0], te.shape[0]
    radii = torch.exp(torch.empty(n_objects, device=dev, dtype=torch.float64).uniform_(
        float(np.log(r_lo)), float(np.log(r_hi)), generator=g))
    R = _rotations(g, n_objects, dev)
    if centers is None:
        centers = torch.rand((n_objects, 3), generator=g, device=dev, dtype=torch.float64) * world
    else:
        centers = centers.to(device=dev, dtype=torch.float64)
    p = torch.einsum("nvk,njk->nvj", tv[None] * radii[:, None, None], R) + centers[:, None, :]
    V = p.to(torch.float32).reshape(-1, 3).contiguous()
    base = (torch.arange(n_objects, device=dev, dtype=torch.int64) * nv)
    I = (tf[None] + base[:, None, None]).reshape(-1, 3).to(torch.int32).contiguous()
    T = torch.arange(n_objects, device=dev, dtype=torch.int32).repeat_interleave(nf).contiguous()
    ei = (te[None] + base[:, None, None]).reshape(-1, 2)
    starts = V[ei[:, 0]].contiguous()
    ends = V[ei[:, 1]].contiguous()
    nE = n_objects * ne
    offsets = torch.arange(nE, device=dev, dtype=torch.int32)
    counts = torch.ones(nE, device=dev, dtype=torch.int32)
    sources = torch.arange(n_objects, device=dev, dtype=torch.int32).repeat_interleave(ne).contiguous()
    return DeviceGeometry.from_tensors(V, I, T, edges=(starts, ends, offsets, counts, sources))


def mesh_points(dg: DeviceGeometry, n: int, seed: int, frac_snapped: float = 0.2, pad: float = 0.25,
                device="cuda") -> torch.Tensor:
    """n points uniform in the padded bounds of the mesh; a share placed exactly on
    vertices, on edges (rounded convex combinations) and on faces."""
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    lo = dg.V.min(dim=0).values - pad
    hi = dg.V.max(dim=0).values + pad
    pts = lo + torch.rand((n, 3), generator=g, device=dev) * (hi - lo)
    k = int(n * frac_snapped)
    if k and dg.nF:
        tri = dg.I[torch.randint(0, dg.nF, (k,), generator=g, device=dev)].long()
        a, b, c = dg.V[tri[:, 0]].double(), dg.V[tri[:, 1]].double(), dg.V[tri[:, 2]].double()
        which = torch.randint(0, 3, (k, 1), generator=g, device=dev)
        w = torch.rand((k, 1), generator=g, device=dev, dtype=torch.float64)
        u = -torch.log(torch.rand((k, 3), generator=g, device=dev, dtype=torch.float64).clamp_min(1e-300))
        u = u / u.sum(dim=1, keepdim=True)
        snap = torch.where(which == 0, a, torch.where(which == 1, a + w * (b - a),
                                                      u[:, :1] * a + u[:, 1:2] * b + u[:, 2:] * c))
        idx = torch.randperm(n, generator=g, device=dev)[:k]
        pts[idx] = snap.to(torch.float32)
    return pts.contiguous()


def to_host_geometry(dg: DeviceGeometry):
    """Host copy (for the oracle on small cases)."""
    from .formats import Edges, Geometry
    V = dg.V.cpu().numpy()
    I = dg.I.cpu().numpy().view(np.uint32)
    T = dg.T.cpu().numpy()
    edges = None
    if dg.edges is not None:
        s, e, o, c, src = [t.cpu().numpy() for t in dg.edges]
        edges = Edges(s, e, o, c, src)
    return Geometry(V, I, T, total_triangles=len(I), edges=edges)


def concat(parts) -> DeviceGeometry:
    """One set from several (object ids and vertex indices offset; edges included)."""
    Vs, Is, Ts, E = [], [], [], [[], [], [], [], []]
    voff = ooff = eoff = soff = 0
    for g in parts:
        Vs.append(g.V)
        Is.append(g.I + voff)
        Ts.append(g.T + ooff)
        if g.edges is not None:
            s, e, o, c, src = g.edges
            E[0].append(s)
            E[1].append(e)
            E[2].append(o + soff)
            E[3].append(c)
            E[4].append(src + ooff)
            soff += int(src.shape[0])
        voff += g.nV
        ooff += int(g.T.max().item()) + 1 if g.nF else 0
    edges = tuple(torch.cat(x) for x in E) if E[0] else None
    return DeviceGeometry.from_tensors(torch.cat(Vs), torch.cat(Is), torch.cat(Ts), edges=edges)


def mixture_centers(n: int, k: int, world: float, seed: int, device="cuda") -> torch.Tensor:
    """n centres from a Gaussian mixture of k components (means uniform in the world,
    sigma log-uniform in [world/200, world/5], weights Dirichlet(1)), clipped to the world."""
    dev = torch.device(device)
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    means = torch.rand((k, 3), generator=g, dtype=torch.float64) * world
    sig = torch.exp(torch.empty(k, dtype=torch.float64).uniform_(float(np.log(world / 200)),
                                                                  float(np.log(world / 5)), generator=g))
    w = -torch.log(torch.rand(k, generator=g, dtype=torch.float64).clamp_min(1e-12))
    comp = torch.multinomial(w / w.sum(), n, replacement=True, generator=g)
    c = means[comp] + torch.randn((n, 3), generator=g, dtype=torch.float64) * sig[comp, None]
    return c.clamp(0.0, world).to(dev)


def intersection_sets(n: int, seed: int, world: float = 2000.0, levels=(1, 2, 3, 4, 5), r_lo: float = 0.2,
                      r_hi: float = 20.0, frac_inside: float = 0.05, device="cuda"):
    """The full-intersection configuration: n objects per set, icospheres whose level is
    drawn uniformly from `levels` (triangle counts log-uniform), radii log-uniform in
    [r_lo, r_hi], centres uniform in [0, world]^3.  A share frac_inside of B is placed
    strictly inside random A objects: radius 0.10..0.35 of the A radius, centre offset
    below 0.9 (0.75 R_A - r_B), so the whole object stays within 0.8 R_A, inside the
    inscribed sphere of any icosphere of level >= 1 (0.94 R).  Returns (A, B, planted),
    planted = list of (a, b) object ids."""
    rng = np.random.default_rng(seed)
    dev = torch.device(device)

    def draw(k):
        lv = rng.choice(np.asarray(levels), size=k)
        r = np.exp(rng.uniform(np.log(r_lo), np.log(r_hi), size=k))
        c = rng.uniform(0.0, world, size=(k, 3))
        return lv, r, c

    la, ra, ca = draw(n)
    lb, rb, cb = draw(n)
    k_in = int(round(n * frac_inside))
    inside_b = rng.choice(n, size=k_in, replace=False)
    host_a = rng.integers(0, n, size=k_in)
    planted = []
    for b, a in zip(inside_b, host_a):
        rb[b] = ra[a] * rng.uniform(0.10, 0.35)
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        off = rng.uniform(0.0, 1.0) * 0.9 * (0.75 * ra[a] - rb[b])
        cb[b] = ca[a] + v * off
        planted.append((int(a), int(b)))

    def build(lv, r, c, sseed):
        # objects keep their ids: each level's objects are generated together and the
        # vertex/index/edge blocks are reordered back to id order afterwards
        parts, ids = [], []
        for L in sorted(set(lv.tolist())):
            idx = np.nonzero(lv == L)[0]
            g = instanced_set(len(idx), int(L), 1.0, 1.0, 0.0, seed=sseed + int(L), device=device,
                              centers=torch.from_numpy(c[idx]))
            # radii: scale each object's vertices about its centre
            nv = g.nV // len(idx)
            cc = torch.from_numpy(c[idx]).to(dev)
            rr = torch.from_numpy(r[idx]).to(dev)
            Vd = g.V.double().view(len(idx), nv, 3)
            Vd = (Vd - cc[:, None, :]) * rr[:, None, None] + cc[:, None, :]
            V = Vd.to(torch.float32).reshape(-1, 3)
            s, e, o, cnt, src = g.edges
            ne = s.shape[0] // len(idx)
            s = ((s.double().view(len(idx), ne, 3) - cc[:, None, :]) * rr[:, None, None] + cc[:, None, :]) \
                .to(torch.float32).reshape(-1, 3)
            e = ((e.double().view(len(idx), ne, 3) - cc[:, None, :]) * rr[:, None, None] + cc[:, None, :]) \
                .to(torch.float32).reshape(-1, 3)
            idmap = torch.from_numpy(idx.astype(np.int32)).to(dev)
            T = idmap[g.T.long()]
            src = idmap[src.long()]
            parts.append(DeviceGeometry.from_tensors(V, g.I, T, edges=(s, e, o, cnt, src)))
            ids.append(idx)
        # concatenate without renumbering objects
        Vs, Is, Ts, E = [], [], [], [[], [], [], [], []]
        voff = soff = 0
        for g in parts:
            Vs.append(g.V)
            Is.append(g.I + voff)
            Ts.append(g.T)
            s, e, o, cnt, src = g.edges
            E[0].append(s)
            E[1].append(e)
            E[2].append(o + soff)
            E[3].append(cnt)
            E[4].append(src)
            soff += int(src.shape[0])
            voff += g.nV
        return DeviceGeometry.from_tensors(torch.cat(Vs), torch.cat(Is), torch.cat(Ts),
                                           edges=tuple(torch.cat(x) for x in E))

    A = build(la, ra, ca, 100 * seed + 1)
    B = build(lb, rb, cb, 100 * seed + 51)
    return A, B, planted
