"""The reference's own CUDA kernels, loaded from the cubins oracle/ref_build.py compiles
(TEST INFRASTRUCTURE: only tests/ use this module).

The cubins hold the device code of query/src/cuda/estimated_overlap.cu,
estimated_intersection.cu, mesh_query_deduplication.cu and result_compaction.cu, compiled
unmodified.  Their kernels have C++ linkage, so they are looked up by their Itanium
mangled names (spelled out below from the kernels' signatures) and launched through the
CUDA driver API, in the primary context that PyTorch uses, with the block sizes the
reference's host functions use (256 threads).
"""
from __future__ import annotations

import ctypes
import os

from . import ref_build

# name in the reference -> (cubin, mangled symbol)
KERNELS = {
    "estimateSelectivityKernel@overlap": ("estimated_overlap", "_Z25estimateSelectivityKernelPK8GridCellS1_Pfifff"),
    "estimateSelectivityKernel@intersection": ("estimated_intersection",
                                               "_Z25estimateSelectivityKernelPK8GridCellS1_Pfifff"),
    "compact_hash_pairs_kernel": ("mesh_query_deduplication", "_Z25compact_hash_pairs_kernelPKyyP15MeshQueryResultPii"),
    "pairs_to_keys_kernel": ("mesh_query_deduplication", "_Z20pairs_to_keys_kernelPK15MeshQueryResultPyx"),
    "keys_to_pairs_kernel": ("mesh_query_deduplication", "_Z20keys_to_pairs_kernelPKyP15MeshQueryResultx"),
    "count_hits_kernel": ("result_compaction", "_Z17count_hits_kernelPK9RayResultiPi"),
    "compact_hits_kernel": ("result_compaction", "_Z19compact_hits_kernelPK9RayResultPS_iPi"),
}

_cu = None
_modules = {}


def available() -> bool:
    return all(os.path.exists(ref_build.cubin_path(n)) for n in ref_build.CUDA_SOURCES)


def _driver():
    global _cu
    if _cu is None:
        cu = ctypes.CDLL("libcuda.so.1")
        cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                 ctypes.POINTER(ctypes.c_void_p),
                                                                                 ctypes.c_void_p]
        cu.cuCtxSynchronize.argtypes = []
        _cu = cu
    return _cu


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what}: CUresult {rc}")


def kernel(name: str):
    """A launcher for one reference kernel: fn(grid, block, *args) with ctypes arguments."""
    import torch
    torch.cuda.init()
    torch.empty(1, device="cuda")  # the primary context is current on this thread
    cubin, symbol = KERNELS[name]
    if cubin not in _modules:
        data = open(ref_build.cubin_path(cubin), "rb").read()
        buf = ctypes.create_string_buffer(data, len(data))
        mod = ctypes.c_void_p()
        _check(_driver().cuModuleLoadData(ctypes.byref(mod), ctypes.cast(buf, ctypes.c_void_p)), "cuModuleLoadData")
        _modules[cubin] = (mod, buf)
    fn = ctypes.c_void_p()
    _check(_driver().cuModuleGetFunction(ctypes.byref(fn), _modules[cubin][0], symbol.encode()),
           f"cuModuleGetFunction {symbol}")

    def launch(grid: int, block: int, *args):
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        _check(_driver().cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, None, ptrs, None), f"cuLaunchKernel {name}")
        _check(_driver().cuCtxSynchronize(), f"{name}")

    return launch


def ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())
