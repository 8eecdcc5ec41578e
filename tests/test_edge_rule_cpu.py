"""The oracle's edge loop and parity loop against the reference's loops run literally.

mesh_overlap_edges.cu:114-178 traces an edge again and again, each time for the closest
crossing beyond t_min, which starts at 1e-6 and steps to t + 1e-6 (t + 2e-4 when that float
sum does not exceed t) after each hit, at most 100 times; raytracer_containment's edge
check steps to the next float instead, at most 256 times (mesh_containment.cu:99-170).
`edge_cases.reference_loop` does exactly that, trace by trace, on each edge's crossing
list; the oracle walks the sorted list instead.  raytracing.cu:22-77 counts parity with
the t + 1e-6 step and a 10000-iteration cap: when the step cannot advance (t >= 32) every
remaining trace finds the same hit, so the count ends at 10000 (even)."""
import numpy as np
import pytest

import edge_cases as ec
from oracle import bind
from rayspace3d_gb300 import synth


@pytest.mark.parametrize("name", sorted(ec.CASES))
def test_oracle_edge_walk_is_the_reference_loop(name):
    A, B, segs = ec.CASES[name]()
    for max_hits, next_float in ec.RULES:
        got = bind.edge_join(segs, B.vertices, B.indices, B.tri2obj, max_hits=max_hits, next_float=next_float)
        np.testing.assert_array_equal(got, ec.loop_keys(segs, B, False, max_hits, next_float))
        got = bind.overlap_join(A, B, max_hits=max_hits, next_float=next_float)
        np.testing.assert_array_equal(got, ec.loop_pairs(A, B, max_hits, next_float))


@pytest.mark.parametrize("name", sorted(ec.CASES))
def test_overlap_rule_drops_crossings(name):
    # Every case loses pairs to the cap or the step: the cases exercise the rule.
    A, B, segs = ec.CASES[name]()
    taken = bind.edge_join(segs, B.vertices, B.indices, B.tri2obj, max_hits=100)
    assert len(taken) < len(ec.loop_keys(segs, B, every=True))
    assert set(taken.tolist()) <= set(ec.loop_keys(segs, B, every=True).tolist())


def test_slab_stack_cap_counts():
    # 240 crossings per direction: 100 traces take the 50 slabs nearest the segment's start.
    A, B, segs = ec.slab_stack()
    keys = bind.edge_join(segs, B.vertices, B.indices, B.tri2obj, max_hits=100)
    fwd = sorted(int(k & 0xffffffff) for k in keys if k >> 32 == 0)
    back = sorted(int(k & 0xffffffff) for k in keys if k >> 32 == 1)
    assert fwd == list(range(50)) and back == list(range(70, 120))
    assert len(bind.edge_join(segs, B.vertices, B.indices, B.tri2obj, max_hits=0)) == 100  # <= 0 means 100


def tall_box_points():
    g = synth.box_set([((0.0, 0.0, 0.0), (1.0, 1.0, 100.0))], edges=False)
    pts = np.array([[0.3, 0.6, 40.0],    # inside, exit at t = 60: the step is stuck, count 10000
                    [0.3, 0.6, 90.0],    # inside, exit at t = 10
                    [0.3, 0.6, -50.0],   # below: crossings at t = 50 and 150
                    [0.3, 0.6, 67.9]],   # inside, exit at t = 32.1
                   np.float32)
    return g, pts, [-1, 0, -1, -1]


def test_pim_iteration_cap():
    g, pts, want = tall_box_points()
    assert bind.pim(g.vertices, g.indices, g.tri2obj, pts).tolist() == want
    assert bind.pim(g.vertices, g.indices, g.tri2obj, pts, use_bvh=False).tolist() == want
