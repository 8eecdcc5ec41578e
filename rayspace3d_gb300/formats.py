"""Byte formats of the RaySpace3D query path, restated in numpy.

* ``.pre`` geometry files, version 2 (``common/include/BinaryIO.h:14-33`` header and
  grid params, ``:35-102`` writer, ``:104-180`` reader) and the version-1 layout of the
  bundled fixture (48-byte header, no edge payload).
* WKT / bare ``x y z`` point files (``query/src/runtime/PointIO.cpp:32-92``).
* The phase-timing JSON (``query/src/timer.cpp:124-192``).

The C++ executables carry their own reader (``rayspace3d_gb300/host/common/cli_common.cpp``); this
module is the Python-side equivalent used by the Python API, the synthetic generator,
the tests and the benchmark.
"""
from __future__ import annotations

import dataclasses
import json
import struct
from typing import Dict, Optional

import numpy as np

PRE_MAGIC = 0x52334442  # "R3DB"
PRE_VERSION = 2
GRID_CELL_DTYPE = np.dtype([("CenterCount", "<u4"), ("TouchCount", "<u4"),
                            ("AvgSizeMean", "<f4"), ("VolRatio", "<f4")])
_HDR_V2 = struct.Struct("<IIQQQQQQBB6x")  # 64 bytes
_HDR_V1 = struct.Struct("<IIQQQQB7x")     # 48 bytes
_GRID = struct.Struct("<3f3f3I4x")        # 40 bytes


@dataclasses.dataclass
class Grid:
    min_bound: np.ndarray          # float32[3]
    max_bound: np.ndarray          # float32[3]
    resolution: np.ndarray         # uint32[3]
    cells: np.ndarray              # GRID_CELL_DTYPE[res^3], index (z*R+y)*R+x


@dataclasses.dataclass
class Edges:
    starts: np.ndarray             # float32[E,3]
    ends: np.ndarray               # float32[E,3]
    offsets: np.ndarray            # int32[E]
    counts: np.ndarray             # int32[E]
    sources: np.ndarray            # int32[S]


@dataclasses.dataclass
class Geometry:
    vertices: np.ndarray           # float32[V,3]
    indices: np.ndarray            # uint32[F,3]
    tri2obj: np.ndarray            # int32[F]
    total_triangles: int = 0
    edges: Optional[Edges] = None
    grid: Optional[Grid] = None

    @property
    def num_objects(self) -> int:
        return int(self.tri2obj.max()) + 1 if self.tri2obj.size else 0


def write_pre(path: str, g: Geometry) -> None:
    """Write a version-2 ``.pre`` file (BinaryIO.h:35-102 layout, zeroed padding)."""
    V = np.ascontiguousarray(g.vertices, dtype="<f4").reshape(-1, 3)
    I = np.ascontiguousarray(g.indices, dtype="<u4").reshape(-1, 3)
    T = np.ascontiguousarray(g.tri2obj, dtype="<i4").reshape(-1)
    e = g.edges
    has_edges = e is not None and len(e.starts) > 0
    has_grid = g.grid is not None
    hdr = _HDR_V2.pack(PRE_MAGIC, PRE_VERSION, len(V), len(I), len(T),
                       len(e.starts) if has_edges else 0,
                       len(e.sources) if has_edges else 0,
                       int(g.total_triangles or len(I)), int(has_grid), int(has_edges))
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(V.tobytes())
        f.write(I.tobytes())
        f.write(T.tobytes())
        if has_edges:
            f.write(np.ascontiguousarray(e.starts, dtype="<f4").tobytes())
            f.write(np.ascontiguousarray(e.ends, dtype="<f4").tobytes())
            f.write(np.ascontiguousarray(e.offsets, dtype="<i4").tobytes())
            f.write(np.ascontiguousarray(e.counts, dtype="<i4").tobytes())
            f.write(np.ascontiguousarray(e.sources, dtype="<i4").tobytes())
        if has_grid:
            gr = g.grid
            f.write(_GRID.pack(*[float(x) for x in gr.min_bound], *[float(x) for x in gr.max_bound],
                               *[int(x) for x in gr.resolution]))
            f.write(np.ascontiguousarray(gr.cells, dtype=GRID_CELL_DTYPE).tobytes())


class PreFormatError(ValueError):
    pass


def read_pre(path: str) -> Geometry:
    """Read a ``.pre`` file of version 2 (BinaryIO.h:104-180) or version 1 (48-byte header).

    Raises PreFormatError on a bad magic, an unknown version or a truncated file.
    """
    buf = open(path, "rb").read()
    if len(buf) < 8:
        raise PreFormatError(f"{path}: truncated header")
    magic, version = struct.unpack_from("<II", buf, 0)
    if magic != PRE_MAGIC:
        raise PreFormatError(f"{path}: magic mismatch 0x{magic:08x}")
    if version == 2:
        if len(buf) < _HDR_V2.size:
            raise PreFormatError(f"{path}: truncated header")
        (_, _, nV, nI, nM, nE, nES, total, has_grid, has_edges) = _HDR_V2.unpack_from(buf, 0)
        pos = _HDR_V2.size
    elif version == 1:
        if len(buf) < _HDR_V1.size:
            raise PreFormatError(f"{path}: truncated header")
        (_, _, nV, nI, nM, total, has_grid) = _HDR_V1.unpack_from(buf, 0)
        nE = nES = 0
        has_edges = 0
        pos = _HDR_V1.size
    else:
        raise PreFormatError(f"{path}: unsupported version {version}")

    def take(dtype, count, shape=None):
        nonlocal pos
        nbytes = np.dtype(dtype).itemsize * count
        if pos + nbytes > len(buf):
            raise PreFormatError(f"{path}: truncated payload")
        arr = np.frombuffer(buf, dtype=dtype, count=count, offset=pos).copy()
        pos += nbytes
        return arr.reshape(shape) if shape is not None else arr

    V = take("<f4", 3 * nV, (nV, 3))
    I = take("<u4", 3 * nI, (nI, 3))
    T = take("<i4", nM)
    edges = None
    if has_edges:
        starts = take("<f4", 3 * nE, (nE, 3))
        ends = take("<f4", 3 * nE, (nE, 3))
        offsets = take("<i4", nE)
        counts = take("<i4", nE)
        sources = take("<i4", nES)
        edges = Edges(starts, ends, offsets, counts, sources)
    grid = None
    if has_grid:
        if pos + _GRID.size > len(buf):
            raise PreFormatError(f"{path}: truncated grid header")
        vals = _GRID.unpack_from(buf, pos)
        pos += _GRID.size
        res = np.array(vals[6:9], dtype=np.uint32)
        cells = take(GRID_CELL_DTYPE, int(res[0]) * int(res[1]) * int(res[2]))
        grid = Grid(np.array(vals[0:3], np.float32), np.array(vals[3:6], np.float32), res, cells)
    return Geometry(V, I, T, int(total), edges, grid)


def _fgets_segments(data: bytes):
    """The pieces a C ``fgets(buf, 1024, f)`` loop returns: lines ending at ``\n`` (kept),
    with lines longer than 1023 bytes split into 1023-byte pieces."""
    pos = 0
    n = len(data)
    while pos < n:
        nl = data.find(b"\n", pos)
        end = n if nl < 0 else nl + 1
        while end - pos > 1023:
            yield data[pos:pos + 1023].decode("latin-1")
            pos += 1023
        yield data[pos:end].decode("latin-1")
        pos = end


def read_points(path: str) -> np.ndarray:
    """Parse a point file like PointIO.cpp:33-62: ``POINT``-prefixed lines read three
    floats after the first ``(``; lines starting with a digit or ``-`` are bare
    ``x y z``; blank lines and ``#`` comments are skipped; lines are read in fgets
    pieces of at most 1023 characters.  Returns float32[N,3]."""
    out = []
    with open(path, "rb") as f:
        data = f.read()
    for line in _fgets_segments(data):
        s = line.lstrip(" \t")
        if not s or s[0] in "\r\n#":
            continue
        if s.startswith("POINT"):
            k = s.find("(")
            if k < 0:
                continue
            out.append(_strtof3(s[k + 1:]))
        elif "0" <= s[0] <= "9" or s[0] == "-":
            vals = _strtof3(s)
            if vals is not None and not (vals[0] is None):
                out.append(vals)
    arr = np.array([[0.0 if v is None else v for v in p] for p in out if p is not None], dtype=np.float32)
    return arr.reshape(-1, 3)


def _strtof3(s: str):
    toks = s.replace(")", " ").replace(",", " ").split()
    vals = []
    for t in toks[:3]:
        try:
            vals.append(float(np.float32(float(t))))
        except ValueError:
            vals.append(0.0)
    while len(vals) < 3:
        vals.append(0.0)
    return vals


def write_points_wkt(path: str, pts: np.ndarray) -> None:
    """WKT ``POINT (x y z)`` lines with 9 significant digits (float32 round-trips)."""
    with open(path, "w") as f:
        for x, y, z in np.asarray(pts, dtype=np.float32):
            f.write(f"POINT ({float(x):.9g} {float(y):.9g} {float(z):.9g})\n")


def timing_json(phases, counters: Dict[str, int], total_us: Optional[int]) -> str:
    """Render phases [(name, duration_us)] like PerformanceTimer::writeResultsToFile:
    lowercase ``<name>_<k>`` keys, two-decimal milliseconds, counters, total or null."""
    lines = ["{", '  "phases": {']
    seen: Dict[str, int] = {}
    items = []
    for name, us in phases:
        key = name.lower()
        seen[key] = seen.get(key, 0) + 1
        items.append((f"{key}_{seen[key]}", int(us)))
    for i, (k, us) in enumerate(items):
        lines.append(f'    "{k}": {{')
        lines.append(f'      "duration_us": {us},')
        lines.append(f'      "duration_ms": {us / 1000.0:.2f}')
        lines.append("    }" + ("," if i < len(items) - 1 else ""))
    lines.append("  },")
    lines.append('  "counters": {')
    citems = list(counters.items())
    for i, (k, v) in enumerate(citems):
        lines.append(f'    "{k.lower()}": {int(v)}' + ("," if i < len(citems) - 1 else ""))
    lines.append("  },")
    if total_us is not None and total_us > 0:
        lines += ['  "total": {', f'    "duration_us": {int(total_us)},',
                  f'    "duration_ms": {total_us / 1000.0:.2f}', "  }"]
    else:
        lines.append('  "total": null')
    lines.append("}")
    return "\n".join(lines) + "\n"


def parse_timing_json(text: str) -> dict:
    return json.loads(text)
