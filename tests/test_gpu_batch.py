"""Batched persistent launch (rs_batch_*): point-in-mesh queries of several meshes and
directions and both edge directions of a join in one batch, equal to the oracle; graph
replay, options, the >8-crossing fallback and the autotuner."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import bind
from rayspace3d_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu


class Batch:
    def __init__(self):
        self.L = _lib.load()
        self.h = ctypes.c_void_p()
        assert self.L.rs_batch_create(ctypes.byref(self.h)) == 0
        self.keep = []

    def add_pim(self, bvh, pts, d):
        dp = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda()
        obj = torch.full((len(pts),), 7, dtype=torch.int32, device="cuda")
        ins = torch.full((len(pts),), 7, dtype=torch.uint8, device="cuda")
        idx = ctypes.c_int()
        assert self.L.rs_batch_add_pim(self.h, bvh.handle, dp.data_ptr(), len(pts), *map(float, d), obj.data_ptr(),
                                       ins.data_ptr(), ctypes.byref(idx)) == 0
        self.keep += [dp, obj, ins, bvh]
        return obj, ins

    def add_edges(self, target, src_geom, swap, ps):
        e = src_geom.edge_ptrs()
        assert self.L.rs_batch_add_edges(self.h, target.handle, *e, src_geom.nE, swap, ps.handle, None) == 0
        self.keep += [target, src_geom, ps]

    def run(self, stream=None):
        s = stream or torch.cuda.current_stream()
        assert self.L.rs_batch_submit(self.h, ctypes.c_void_p(s.cuda_stream)) == 0
        st = (ctypes.c_int * 64)()
        rc = self.L.rs_batch_wait(self.h, st)
        return rc

    def close(self):
        self.L.rs_batch_destroy(self.h)


def _workload():
    rng = np.random.default_rng(41)
    meshes, queries = [], []
    g1, p1 = synth.pim_workload(30000, level=3, seed=1)
    meshes.append(g1)
    queries += [(0, p1, (1, 0, 0)), (0, p1[:5000], (0, 0, 1)), (0, p1[:7000], (0.3, -0.4, 0.866))]
    cg = synth.cube_grid(3, 2, 2)
    meshes.append(cg)
    queries += [(1, synth.snapped_points(cg, 20000, rng, frac_snapped=0.2), (0, 1, 0)),
                (1, synth.snapped_points(cg, 3000, rng, frac_snapped=0.5), (0, 0, -1))]
    # a stack of 12 separate slabs: +Z rays from below cross 24 faces (fallback path)
    Vs, Is, Ts = [], [], []
    for k in range(12):
        v, f = synth.cube_mesh((0, 0, 2 * k), (1, 1, 2 * k + 1))
        Vs.append(v)
        Is.append(f + np.uint32(8 * k))
        Ts.append(np.full(12, k, np.int32))
    stack = synth.make_geometry(np.concatenate(Vs), np.concatenate(Is), np.concatenate(Ts), edges=False)
    meshes.append(stack)
    sp = rng.uniform([0.05, 0.05, -1.0], [0.95, 0.95, 24.0], size=(4000, 3)).astype(np.float32)
    queries.append((2, sp, (0, 0, 1)))
    return meshes, queries


def _check_batch(batch_opts=None, autotune=False, repeats=2):
    meshes, queries = _workload()
    dgs = [api.DeviceGeometry(m) for m in meshes]
    bvhs = [api.Bvh(d) for d in dgs]
    A, B = synth.overlap_workload(n_objects=200, level=1, world=10.0, seed=42)
    da, db = api.DeviceGeometry(A), api.DeviceGeometry(B)
    ba, bb = api.Bvh(da), api.Bvh(db)
    ps = api.PairSet(1 << 12)
    b = Batch()
    outs = [b.add_pim(bvhs[m], p, d) for m, p, d in queries]
    b.add_edges(bb, da, 0, ps)
    b.add_edges(ba, db, 1, ps)
    L = b.L
    if batch_opts:
        assert L.rs_batch_set_options(b.h, *batch_opts) == 0
    if autotune:
        leaf, ch, sd, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        assert L.rs_batch_autotune(b.h, ctypes.byref(leaf), ctypes.byref(ch), ctypes.byref(sd), ctypes.byref(ms),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        assert leaf.value in (2, 4, 8, 16) and ch.value in (32, 64, 128) and sd.value in (32, 64)
        assert ms.value > 0
    want_pairs = bind.overlap_join(A, B)
    for rep in range(repeats):
        ps.clear()
        for o, i in outs:
            o.fill_(7)
            i.fill_(7)
        assert b.run() == 0
        for (m, p, d), (o, i) in zip(queries, outs):
            g = meshes[m]
            want = bind.pim(g.vertices, g.indices, g.tri2obj, p, direction=d)
            np.testing.assert_array_equal(o.cpu().numpy(), want)
            np.testing.assert_array_equal(i.cpu().numpy().astype(bool), want >= 0)
        np.testing.assert_array_equal(np.sort(ps.finalize().cpu().numpy().astype(np.uint64)), want_pairs)
    b.close()


def test_batch_matches_oracle_and_replays(cuda):
    _check_batch()


@pytest.mark.parametrize("opts", [(32, 32, 0), (128, 64, 1), (4096, 64, 1)])
def test_batch_options(cuda, opts):
    _check_batch(opts, repeats=1)


def test_batch_autotune(cuda):
    _check_batch(autotune=True, repeats=1)
