"""rs_pim_noalloc: point-in-mesh for callers that cannot allocate device memory.

Such callers (services whose own allocator has reserved the whole GPU, hosts with a fixed
device-memory budget checked per request) get the same answers as rs_pim from a fixed
scratch array inside the library.  These tests call the entry point through the C ABI
and compare it with rs_pim / rs_pim_filtered bit for bit (the tolerance of every
integer output in this suite), on two calls in a row so that the shared scratch left
over from one call cannot leak into the next; they also check that the call requests no
allocation from the library's memory pool (rs_alloc_count, which rs_pim does move) and
compare its answers with the CPU oracle.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 20


def _noalloc(bvh, pts, direction, filtered):
    n = int(pts.shape[0])
    obj = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    inside = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    L = _lib.load()
    before = L.rs_alloc_count()
    st = L.rs_pim_noalloc(bvh.handle, pts.data_ptr(), n, float(direction[0]), float(direction[1]),
                          float(direction[2]), obj.data_ptr(), inside.data_ptr(), int(filtered),
                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "rs_pim_noalloc")
    assert L.rs_alloc_count() == before, "rs_pim_noalloc requested a device allocation"
    torch.cuda.synchronize()
    return obj.cpu().numpy(), inside.cpu().numpy()


def _existing(bvh, pts, direction, filtered):
    L = _lib.load()
    before = L.rs_alloc_count()
    obj, inside = api.point_in_mesh(bvh, pts, direction=direction, filtered=filtered)
    torch.cuda.synchronize()
    assert L.rs_alloc_count() > before  # the counter sees the allocating entry point's scratch
    return obj.cpu().numpy(), inside.cpu().numpy()


def _nested_spheres(k=12):
    v, f = synth.icosphere(2)
    Vs, Is, Ts = [], [], []
    for j in range(k):
        Vs.append((v * (1.0 + 0.06 * j)).astype(np.float32))
        Is.append(f + np.uint32(len(v) * j))
        Ts.append(np.full(len(f), j, np.int32))
    return synth.make_geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts), edges=False)


@pytest.mark.parametrize("direction,filtered", [((0.0, 0.0, 1.0), False), ((0.0, 0.0, 1.0), True),
                                                ((1.0, 0.0, 0.0), False), ((0.3, -0.4, 0.866), False)])
def test_noalloc_matches_rs_pim_two_calls(cuda, direction, filtered):
    g = _nested_spheres()  # rays from the middle cross more than 8 surfaces: exercises the overflow list
    dg = api.DeviceGeometry(g)
    rng = np.random.default_rng(21)
    for call in range(2):
        n = 50_000 if call == 0 else 20_011
        pts = torch.from_numpy(rng.uniform(-2.2, 2.2, size=(n, 3)).astype(np.float32)).cuda()
        # fresh handle for the first call (no column grid yet) and a reused one afterwards
        bvh = api.Bvh(dg) if call == 0 else bvh_keep
        got = _noalloc(bvh, pts, direction, filtered)
        want = _existing(bvh, pts, direction, filtered)
        assert np.array_equal(got[0], want[0]), f"call {call}: {(got[0] != want[0]).sum()} object mismatches"
        assert np.array_equal(got[1], want[1]), f"call {call}: inside bits differ"
        if call == 0:
            ref = bind.pim(g.vertices, g.indices, g.tri2obj, pts.cpu().numpy(), direction=direction, filtered=filtered)
            assert np.array_equal(got[0], ref), f"{(got[0] != ref).sum()} mismatches against the oracle"
        bvh_keep = bvh
        # after rs_pim built the column grid (axis-aligned rays) the next no-alloc call uses it
        got2 = _noalloc(bvh, pts, direction, filtered)
        assert np.array_equal(got2[0], want[0]) and np.array_equal(got2[1], want[1])


def test_noalloc_rejects_more_than_capacity(cuda):
    g, _ = synth.pim_workload(10, level=1)
    bvh = api.Bvh(api.DeviceGeometry(g))
    dummy = torch.zeros(3, dtype=torch.float32, device="cuda")
    st = _lib.load().rs_pim_noalloc(bvh.handle, dummy.data_ptr(), MAX_POINTS + 1, 0.0, 0.0, 1.0, None, None, 0,
                                    None)
    assert st == _lib.RS_ERR_TOO_LARGE
    assert "capacity" in _lib.status_string(st)
