"""The engine against the reference's own CUDA kernels, compiled unmodified from
query/src/cuda/*.cu into cubins (oracle/ref_build.py) and launched with the reference's
launch shapes (oracle/ref_cuda.py):

* estimateSelectivityKernel (estimated_overlap.cu:8-41, estimated_intersection.cu:8-43):
  every per-cell float equals rs_estimate_grid_cells' bit for bit, and rs_estimate_grid's
  FP64 sum equals the FP64 sum of the reference's cells to 1e-12 relative (summation
  order).  The reference sums those floats with thrust::reduce<float> in its own order;
  the engine keeps FP64, so the reported raw estimate can differ in the float's last bits.
* compact_hash_pairs_kernel (mesh_query_deduplication.cu:31-51): the same pair set as the
  engine's compact_hash_table_pairs and rs_pairset_finalize, and the same count when the
  output is too small.
* pairs_to_keys_kernel / keys_to_pairs_kernel (mesh_query_deduplication.cu:17-29): the key
  layout (id1 << 32 | id2) the engine uses.
* count_hits_kernel / compact_hits_kernel (result_compaction.cu:5-21): the same count and
  the same hit set as count_hits_gpu / compact_hits_gpu and rs_compact_hits.

The sort, unique, scan and reduce steps of those files are thrust (CCCL) library calls,
pinned through numpy's sort/unique/cumsum in test_gpu_parity.py."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import ref_cuda
from rayspace3d_gb300 import _lib, api, synth

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(), reason="reference cubins not built on this machine")]


def _grids(world, seed, res=64):
    A, B = synth.overlap_workload(n_objects=3000, level=2, world=world, seed=seed, grid_resolution=res)
    return A.grid, B.grid


@pytest.mark.parametrize("which", ["overlap", "intersection"])
@pytest.mark.parametrize("world,eps,gamma", [(80.7, 0.001, 0.8), (300.0, 0.01, 1.3), (80.7, 0.0, 0.5)])
def test_estimator_cells_equal_reference_kernel(cuda, which, world, eps, gamma):
    ga, gb = _grids(world, 3)
    n = len(ga.cells)
    da = torch.from_numpy(np.ascontiguousarray(ga.cells).view(np.uint8)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(gb.cells).view(np.uint8)).cuda()
    cv = float(api.cell_volume(ga))
    ref = torch.empty(n, dtype=torch.float32, device="cuda")
    k = ref_cuda.kernel(f"estimateSelectivityKernel@{which}")
    k((n + 255) // 256, 256, ref_cuda.ptr(da), ref_cuda.ptr(db), ref_cuda.ptr(ref), ctypes.c_int(n),
      ctypes.c_float(cv), ctypes.c_float(eps), ctypes.c_float(gamma))
    got = torch.empty(n, dtype=torch.float32, device="cuda")
    L = _lib.load()
    _lib.check(L.rs_estimate_grid_cells(da.data_ptr(), db.data_ptr(), n, cv, eps, gamma, got.data_ptr(), None),
               "rs_estimate_grid_cells")
    r, g = ref.cpu().numpy(), got.cpu().numpy()
    assert (r > 0).sum() > 100
    bad = np.nonzero(r.view(np.uint32) != g.view(np.uint32))[0]
    assert len(bad) == 0, f"{len(bad)} cells differ, first {bad[:5]}: {r[bad[:5]]} vs {g[bad[:5]]}"
    raw = ctypes.c_double()
    _lib.check(L.rs_estimate_grid(da.data_ptr(), db.data_ptr(), n, cv, eps, gamma, ctypes.byref(raw), None, None),
               "rs_estimate_grid")
    want = float(np.sum(r.astype(np.float64)))
    assert abs(raw.value - want) <= 1e-12 * abs(want)


def _table(rng, cap, n_keys):
    slots = np.full(cap, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    keys = np.unique((rng.integers(0, 50_000, n_keys).astype(np.uint64) << np.uint64(32)) |
                     rng.integers(0, 50_000, n_keys).astype(np.uint64))
    pos = rng.choice(cap, size=len(keys), replace=False)
    slots[pos] = keys
    return slots, np.sort(keys)


@pytest.mark.parametrize("cap,n_keys", [(4096, 1000), (1 << 20, 300_000), (1 << 20 | 1, 5)])
def test_hash_compaction_equals_reference_kernel(cuda, cap, n_keys):
    rng = np.random.default_rng(cap + n_keys)
    slots, keys = _table(rng, cap, n_keys)
    d_slots = torch.from_numpy(slots.view(np.int64)).cuda()
    out = torch.zeros(2 * len(keys) + 2, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    k = ref_cuda.kernel("compact_hash_pairs_kernel")
    k((cap + 255) // 256, 256, ref_cuda.ptr(d_slots), ctypes.c_ulonglong(cap), ref_cuda.ptr(out), ref_cuda.ptr(cnt),
      ctypes.c_int(len(keys) + 1))
    m = int(cnt.item())
    pairs = out.cpu().numpy()[:2 * m].reshape(-1, 2).astype(np.int64)
    ref_keys = np.sort(((pairs[:, 0] << 32) | pairs[:, 1]).astype(np.uint64))
    np.testing.assert_array_equal(ref_keys, keys)
    mine = torch.zeros_like(out)
    c2 = _lib.load().compact_hash_table_pairs(d_slots.data_ptr(), cap, mine.data_ptr(), len(keys) + 1)
    assert c2 == m
    p2 = mine.cpu().numpy()[:2 * c2].reshape(-1, 2).astype(np.int64)
    np.testing.assert_array_equal(np.sort(((p2[:, 0] << 32) | p2[:, 1]).astype(np.uint64)), keys)
    # output smaller than the count: both report the capped count
    cnt.zero_()
    small = max(1, len(keys) // 3)
    k((cap + 255) // 256, 256, ref_cuda.ptr(d_slots), ctypes.c_ulonglong(cap), ref_cuda.ptr(out), ref_cuda.ptr(cnt),
      ctypes.c_int(small))
    assert min(int(cnt.item()), small) == _lib.load().compact_hash_table_pairs(d_slots.data_ptr(), cap,
                                                                              mine.data_ptr(), small)


def test_pair_key_layout_equals_reference_kernels(cuda):
    rng = np.random.default_rng(9)
    n = 100_003
    pairs = rng.integers(0, 2 ** 31 - 1, size=(n, 2)).astype(np.int32)
    dp = torch.from_numpy(pairs).cuda()
    keys = torch.empty(n, dtype=torch.int64, device="cuda")
    ref_cuda.kernel("pairs_to_keys_kernel")((n + 255) // 256, 256, ref_cuda.ptr(dp), ref_cuda.ptr(keys),
                                           ctypes.c_longlong(n))
    want = (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint64)
    np.testing.assert_array_equal(keys.cpu().numpy().view(np.uint64), want)
    back = torch.empty_like(dp)
    ref_cuda.kernel("keys_to_pairs_kernel")((n + 255) // 256, 256, ref_cuda.ptr(keys), ref_cuda.ptr(back),
                                           ctypes.c_longlong(n))
    np.testing.assert_array_equal(back.cpu().numpy(), pairs)


def test_hit_compaction_equals_reference_kernels(cuda):
    g, pts = synth.pim_workload(200_000, level=3, seed=4)
    bvh = api.Bvh(api.DeviceGeometry(g))
    obj, _ = api.point_in_mesh(bvh, torch.from_numpy(pts).cuda())
    n = len(pts)
    rr = torch.stack([torch.arange(n, dtype=torch.int32, device="cuda"), obj], dim=1).contiguous()  # RayResult[n]
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref_cuda.kernel("count_hits_kernel")((n + 255) // 256, 256, ref_cuda.ptr(rr), ctypes.c_int(n), ref_cuda.ptr(cnt))
    L = _lib.load()
    assert int(cnt.item()) == L.count_hits_gpu(rr.data_ptr(), n) == int((obj >= 0).sum().item())
    out = torch.zeros_like(rr)
    cnt.zero_()
    ref_cuda.kernel("compact_hits_kernel")((n + 255) // 256, 256, ref_cuda.ptr(rr), ref_cuda.ptr(out),
                                          ctypes.c_int(n), ref_cuda.ptr(cnt))
    m = int(cnt.item())
    ref_rows = out.cpu().numpy()[:m]
    ref_rows = ref_rows[np.argsort(ref_rows[:, 0])]
    mine = torch.zeros_like(rr)
    h = ctypes.c_int()
    L.compact_hits_gpu(rr.data_ptr(), mine.data_ptr(), n, ctypes.byref(h))
    assert h.value == m
    my_rows = mine.cpu().numpy()[:m]
    np.testing.assert_array_equal(my_rows[np.argsort(my_rows[:, 0])], ref_rows)
    # the engine's ordered compaction gives the same rows, ascending
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    objs = torch.empty(n, dtype=torch.int32, device="cuda")
    c = ctypes.c_uint64()
    _lib.check(L.rs_compact_hits(obj.data_ptr(), n, ids.data_ptr(), objs.data_ptr(), n, ctypes.byref(c), None),
               "rs_compact_hits")
    np.testing.assert_array_equal(np.stack([ids.cpu().numpy()[:c.value], objs.cpu().numpy()[:c.value]], 1), ref_rows)
