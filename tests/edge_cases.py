"""Geometries on which the reference's edge loop (mesh_overlap_edges.cu:114-178) takes
fewer crossings than a ray meets: more crossings than the 100-iteration cap, and faces
of two objects closer than the 1e-6 (or, beyond t = 32, 2e-4) step along an edge.

Each case gives (A, B, segs): A is a long thin box (object 0) crossing B's boxes, and
segs an edge payload of single segments along A's axis, one per direction, so that the
order in which a segment meets the faces is fixed.  The pairs the reference finds come
from `loop_keys`, which runs the reference's trace loop literally, one closest-hit trace
per iteration, on each segment's list of crossings."""
from __future__ import annotations

import numpy as np

from rayspace3d_gb300 import synth
from rayspace3d_gb300.formats import Edges

# Off the face diagonals of B's boxes (y = +-z for the slabs, y = z and y = 1 - z for the
# unit cubes), so that no edge of B meets A's bar.
_Y, _Z = 0.31, -0.51


def _bar(x0, x1, y=_Y, z=_Z):
    return synth.box_set([((x0, y - 0.01, z - 0.01), (x1, y + 0.01, z + 0.01))])


def segments(segs) -> Edges:
    """Edge payload of (start, end, source objects) segments."""
    starts = np.array([s for s, _, _ in segs], np.float32).reshape(-1, 3)
    ends = np.array([e for _, e, _ in segs], np.float32).reshape(-1, 3)
    counts = np.array([len(src) for _, _, src in segs], np.int32)
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int32)
    sources = np.array([o for _, _, src in segs for o in src], np.int32)
    return Edges(starts, ends, offsets, counts, sources)


def _both_ways(x0, x1, y=_Y, z=_Z):
    return segments([((x0, y, z), (x1, y, z), [0]), ((x1, y, z), (x0, y, z), [1])])


def slab_stack(n=120):
    """n slabs 0.01 thick, 0.05 apart along x, crossed by A's bar (2n crossings per long
    edge): 100 traces reach the 50 slabs nearest to an edge's start."""
    B = synth.box_set([((0.05 * i, -1.0, -1.0), (0.05 * i + 0.01, 1.0, 1.0)) for i in range(n)])
    x0, x1 = -0.5, 0.05 * n + 0.5
    return _bar(x0, x1), B, _both_ways(x0, x1)


def shared_face():
    """Two unit cubes sharing the face x = 1; A's bar runs from inside cube 0 to inside
    cube 1, so its only crossings are the shared face's two coincident triangles, of which
    the loop takes the first in (t, triangle id) order."""
    B = synth.box_set([((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), ((1.0, 0.0, 0.0), (2.0, 1.0, 1.0))])
    y, z = 0.31, 0.61
    return _bar(0.5, 1.5, y, z), B, _both_ways(0.5, 1.5, y, z)


def near_faces(gap=3e-7):
    """Slab 1, `gap` thick, sits `gap` after slab 0's end and `gap` before slab 2; A's bar
    runs from inside slab 0 to inside slab 2.  Every face crossing lies within 1e-6 of the
    first, so the t + 1e-6 step takes only the first slab met; the next-float step takes
    all three."""
    f = np.float32
    x = [f(0.7), f(0.7) + f(gap), f(0.7) + f(2 * gap), f(0.7) + f(3 * gap)]
    B = synth.box_set([((0.5, -1.0, -1.0), (float(x[0]), 1.0, 1.0)),
                       ((float(x[1]), -1.0, -1.0), (float(x[2]), 1.0, 1.0)),
                       ((float(x[3]), -1.0, -1.0), (0.9, 1.0, 1.0))])
    return _bar(0.6, 0.8), B, _both_ways(0.6, 0.8)


def far_faces():
    """Slab 1 (5e-5 thick) between slab 0 and slab 2, 5e-5 apart, near x = 40.5: along an
    edge starting at x = 0 the crossings lie at t > 32, where t + 1e-6 rounds back to t and
    the loop steps by 2e-4, skipping slab 1 and slab 2's face."""
    B = synth.box_set([((40.0, -1.0, -1.0), (40.5, 1.0, 1.0)), ((40.50005, -1.0, -1.0), (40.5001, 1.0, 1.0)),
                       ((40.50015, -1.0, -1.0), (41.5, 1.0, 1.0))])
    return _bar(0.0, 41.0), B, segments([((0.0, _Y, _Z), (41.0, _Y, _Z), [0])])


def deep_stack():
    """slab_stack with 200 slabs: 400 crossings per long edge, more than the 256 one warp
    of the long path collects in one traversal, so the one-thread loop takes them 16 per
    traversal (all 400 under the 1000-trace rule)."""
    return slab_stack(200)


CASES = {"slab_stack": slab_stack, "deep_stack": deep_stack, "shared_face": shared_face, "near_faces": near_faces,
         "far_faces": far_faces}
RULES = [(100, False), (1000, False), (256, True)]


def reference_loop(hits_t, hits_tri, tri2obj, edge_len, max_iters=100, next_float=False):
    """The reference's trace loop, one trace per iteration (mesh_overlap_edges.cu:125-178;
    next_float: mesh_containment.cu:106-170): each trace returns the closest crossing with
    t >= t_min (ties: lowest triangle id), in float32 arithmetic.  Returns the objects of
    the crossings taken, in order."""
    f32 = np.float32
    tmax = f32(f32(edge_len) + f32(1e-6))
    order = sorted(zip(hits_t.tolist(), hits_tri.tolist()))
    t_min = f32(1e-6)
    out = []
    for _ in range(max_iters):
        if t_min > tmax:
            break
        cand = [(t, k) for t, k in order if f32(t) >= t_min]
        if not cand:
            break
        t, k = cand[0]
        t = f32(t)
        out.append(int(tri2obj[k]))
        if next_float:
            nt = np.nextafter(t, tmax, dtype=np.float32)
            if nt <= t:
                nt = f32(t + f32(1e-6))
            if nt <= t_min:
                nt = np.nextafter(t_min, tmax, dtype=np.float32)
            if nt <= t_min:
                break
        else:
            nt = f32(t + f32(1e-6))
            if nt <= t:
                nt = f32(t + f32(2e-4))
        t_min = nt
    return out


def edge_length(s, e):
    f32 = np.float32
    d = [f32(f32(e[k]) - f32(s[k])) for k in range(3)]
    return f32(np.sqrt(f32(f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) + f32(d[2] * d[2]))))


def loop_keys(edges, tgt, swap=False, max_iters=100, next_float=False, every=False):
    """Sorted keys of one edge direction under the reference's loop (every=True: every
    crossing, the rule's counterfactual)."""
    from oracle import bind
    keys = set()
    for i in range(len(edges.starts)):
        t, tri = bind.segment_hits(edges.starts[i], edges.ends[i], tgt.vertices, tgt.indices, tgt.tri2obj)
        if len(t) == 0:
            continue
        if every:
            objs = [int(tgt.tri2obj[k]) for k in tri]
        else:
            objs = reference_loop(t, tri, tgt.tri2obj, edge_length(edges.starts[i], edges.ends[i]), max_iters,
                                  next_float)
        for s_obj in edges.sources[edges.offsets[i]:edges.offsets[i] + edges.counts[i]]:
            for o in objs:
                keys.add((o << 32) | int(s_obj) if swap else (int(s_obj) << 32) | o)
    return np.array(sorted(keys), dtype=np.uint64)


def loop_pairs(A, B, max_iters=100, next_float=False, every=False):
    """The join A x B: A's edges against B as (source, target), B's against A swapped."""
    return np.union1d(loop_keys(A.edges, B, False, max_iters, next_float, every),
                      loop_keys(B.edges, A, True, max_iters, next_float, every)).astype(np.uint64)
